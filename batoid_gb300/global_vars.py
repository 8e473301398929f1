"""Runtime settings mirroring batoid/global_vars.py.

``_batoid_max_threads`` is kept for API compatibility (the GPU path ignores
it); ``_batoid_niter`` caps the Newton iterations of every intersection.
"""
import os

_batoid_max_threads = int(os.environ.get('OMP_NUM_THREADS', 1))
_batoid_niter = 5
