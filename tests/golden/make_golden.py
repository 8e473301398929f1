"""Generate the golden fixtures in tests/golden/ by running the REFERENCE.

Run in a container that has the reference sources and its compiled module
(oracle/Makefile.ref builds oracle/_ref/_batoid*.so from them):

    make -f oracle/Makefile.ref REF=/path/to/reference -j8
    python tests/golden/make_golden.py /path/to/reference   (or BATOID_REF)

Every fixture stores seeded inputs and the reference's outputs for them.
The inputs are regenerated from the same seeds by the tests, so only the
outputs strictly need storing; the inputs are stored too so that a test
can tell an input-generation drift from a compute mismatch.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ref_import import import_reference  # noqa: E402
from batoid_gb300 import workloads as W  # noqa: E402
from batoid_gb300 import zpoly as ZK  # noqa: E402

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "t", "wavelength", "flux", "vignetted", "failed")


def ref_zernike_factory(batoid):
    """A reference PolynomialSurface holding the same Cartesian arrays this
    package builds (GalSim, which the reference's Zernike needs, is absent)."""
    def make(coef, R_outer, R_inner):
        C = ZK.zernike_xy(coef, R_outer, R_inner)
        gx, gy = ZK.grad_xy(C)
        z = batoid.Zernike.__new__(batoid.Zernike)
        z.coef = np.asarray(coef, dtype=float)
        z.R_outer, z.R_inner, z.x_origin, z.y_origin = R_outer, R_inner, 0.0, 0.0
        z._xycoef = np.ascontiguousarray(C)
        z._xycoef_gradx = np.ascontiguousarray(gx)
        z._xycoef_grady = np.ascontiguousarray(gy)
        z._surface = batoid._batoid.CPPPolynomialSurface(
            z._xycoef.ctypes.data, z._xycoef_gradx.ctypes.data, z._xycoef_grady.ctypes.data, 0.0, 0.0,
            C.shape[0], C.shape[1])
        return z
    return make


def rv_to_dict(rv, prefix):
    return {f"{prefix}_{k}": np.array(getattr(rv, k)) for k in FIELDS}


def make_rv(batoid, arrs):
    return batoid.RayVector(*[np.array(a) for a in arrs])


def workload_fixtures(batoid):
    out = {}
    # f/4 paraboloid: full trace and traceFull
    opt = W.paraboloid_optic(batoid)
    arrs = W.paraboloid_rays(4096, seed=57721)
    rv = make_rv(batoid, arrs)
    tf = opt.traceFull(rv)
    for k, v in tf.items():
        out.update(rv_to_dict(v["out"], f"paraboloid_{k}"))
    rv2 = make_rv(batoid, arrs)
    opt.trace(rv2)
    out.update(rv_to_dict(rv2, "paraboloid_final"))
    # sumAmplitude / phase at a few points on the traced rays
    pts = np.array([[0.0, 0.0, 0.0], [1e-5, -2e-5, 0.0], [3e-4, 1e-4, 1e-6]])
    t0 = float(rv2.t[0])
    out["paraboloid_amp_points"] = pts
    out["paraboloid_amp_t0"] = np.array(t0)
    out["paraboloid_sumamp"] = np.array([rv2.sumAmplitude(p, t0) for p in pts])
    out["paraboloid_sumamp_all"] = np.array([rv2.sumAmplitude(p, t0, ignoreVignetted=False) for p in pts])
    out["paraboloid_phase"] = rv2.phase(pts[1], t0)
    out["paraboloid_amplitude"] = rv2.amplitude(pts[1], t0)
    out["paraboloid_pos_at_time"] = rv2.positionAtTime(t0 + 0.01)

    # 12-surface system
    opt = W.tma_optic(batoid, zernike_factory=ref_zernike_factory(batoid))
    arrs = W.tma_rays(2048, seed=8675309)
    rv = make_rv(batoid, arrs)
    tf = opt.traceFull(rv)
    out["tma_names"] = np.array(list(tf.keys()))
    for k, v in tf.items():
        out.update(rv_to_dict(v["out"], f"tma_{k}"))
    return out


def huygens_fixture(batoid):
    """Reference Huygens amplitudes on a small lattice (the per-pixel
    sumAmplitude loop of batoid/analysis.py:296-304)."""
    out = {}
    opt = W.tma_optic(batoid, zernike_factory=ref_zernike_factory(batoid))
    for case, (tx, ty, w, nx, npix) in enumerate([(0.0, 0.0, 500e-9, 64, 24), (0.01, -0.015, 870e-9, 48, 16)]):
        dirCos = batoid.utils.fieldToDirCos(tx, ty)
        rays = batoid.RayVector.asGrid(optic=opt, wavelength=w, dirCos=dirCos, nx=nx)
        opt.trace(rays)
        cridx = (nx // 2) * nx + nx // 2
        point = rays.r[cridx]
        prim = np.array([[2e-6, 0.0], [0.0, 2e-6]])
        lat = batoid.Lattice(np.zeros((npix, npix)), prim)
        xs = lat.coords[..., 0].T + point[0]
        ys = lat.coords[..., 1].T + point[1]
        t0 = rays.t[0]
        amps = np.zeros((npix, npix), dtype=np.complex128)
        for idx in np.ndindex(amps.shape):
            amps[idx] = rays.sumAmplitude(np.array([xs[idx], ys[idx], 0.0]), t0)
        p = f"huy{case}"
        out[f"{p}_params"] = np.array([tx, ty, w, nx, npix])
        out[f"{p}_point"] = point
        out[f"{p}_t0"] = np.array(t0)
        out[f"{p}_amps"] = amps
        out.update(rv_to_dict(rays, f"{p}_rays"))
    return out


def surfaces(batoid, rng):
    """(name, surface) pairs covering every surface kind."""
    zf = ref_zernike_factory(batoid)
    xs = np.linspace(-1.1, 1.1, 40)
    ys = np.linspace(-1.2, 1.2, 44)
    X, Y = np.meshgrid(xs, ys)
    Zt = 0.01 * np.cos(1.3 * X) * np.sin(0.9 * Y) + 0.003 * X * X
    bic = batoid.Bicubic(xs, ys, Zt)
    bic0 = batoid.Bicubic(xs, ys, Zt, nanpolicy='zero')
    zc = np.zeros(23)
    zc[4:] = rng.normal(0, 1e-4, 19)
    return [
        ("plane", batoid.Plane()),
        ("tilted", batoid.Tilted(0.01, -0.02)),
        ("sphere", batoid.Sphere(5.3)),
        ("sphere_neg", batoid.Sphere(-4.1)),
        ("paraboloid", batoid.Paraboloid(3.7)),
        ("quadric", batoid.Quadric(6.1, -0.7)),
        ("quadric_obl", batoid.Quadric(-8.2, 0.4)),
        ("asphere", batoid.Asphere(7.5, -1.1, [1e-4, -2e-5, 3e-7, -1e-8])),
        ("zernike", zf(zc, 1.3, 0.4)),
        ("bicubic", bic),
        ("bicubic_zero", bic0),
        ("sum_asphere_zernike", batoid.Sum([batoid.Asphere(9.0, -0.9, [2e-5, -1e-7]), zf(zc, 1.5, 0.0)])),
        ("sum_quadric_bicubic", batoid.Sum([batoid.Quadric(8.0, -0.5), bic])),
        ("sum_tilted_sphere", batoid.Sum([batoid.Tilted(0.005, 0.003), batoid.Sphere(20.0)])),
    ]


def primitive_fixtures(batoid):
    rng = np.random.default_rng(31415)
    out = {}
    silica = batoid.SellmeierMedium(*W.SILICA)
    vac = batoid.ConstMedium(1.0)
    coat = batoid.SimpleCoating(0.2, 0.7)
    for name, s in surfaces(batoid, rng):
        n = 256
        x = rng.uniform(-0.9, 0.9, n)
        y = rng.uniform(-0.9, 0.9, n)
        out[f"surf_{name}_xy"] = np.stack([x, y])
        out[f"surf_{name}_sag"] = s.sag(x, y)
        out[f"surf_{name}_normal"] = s.normal(x, y)
        # rays from above with mild tilt, some steep ones to fail
        vx = rng.normal(0, 0.1, n)
        vy = rng.normal(0, 0.1, n)
        vx[:12] = rng.uniform(0.9, 0.99, 12)
        vy[:12] = 0.0
        vz = -np.sqrt(1 - vx * vx - vy * vy)
        z = np.full(n, 1.0)
        wl = rng.choice(W.WAVELENGTHS, n)
        origin = rng.normal(0, 0.01, 3)
        rot = batoid.RotX(rng.normal(0, 0.01)) @ batoid.RotY(rng.normal(0, 0.01))
        cs = batoid.CoordSys(origin=origin, rot=rot)
        out[f"surf_{name}_cs"] = np.concatenate([origin, rot.ravel()])
        inputs = (x, y, z, vx, vy, vz, np.zeros(n), wl, np.ones(n), np.zeros(n, bool), np.zeros(n, bool))
        for k, f in enumerate(FIELDS):
            out[f"surf_{name}_in_{f}"] = np.array(inputs[k])
        for op in ("intersect", "reflect", "refract", "reflect_coated", "refract_rev"):
            rv = make_rv(batoid, inputs)
            if op == "intersect":
                s.intersect(rv, coordSys=cs)
            elif op == "reflect":
                s.reflect(rv, coordSys=cs)
            elif op == "reflect_coated":
                s.reflect(rv, coordSys=cs, coating=coat)
            elif op == "refract":
                s.refract(rv, vac, silica, coordSys=cs)
            else:
                # from glass into vacuum at steep incidence: exercises TIR
                rv2 = make_rv(batoid, inputs)
                rv2 = batoid.RayVector(rv2.x, rv2.y, rv2.z, rv2.vx / 1.45, rv2.vy / 1.45, rv2.vz / 1.45,
                                       rv2.t, rv2.wavelength, rv2.flux)
                rv = rv2
                s.refract(rv, silica, vac, coordSys=cs)
            out.update(rv_to_dict(rv, f"surf_{name}_{op}"))
    # obscurations
    pts = rng.uniform(-1.5, 1.5, (2, 5000))
    obscs = {
        "circle": batoid.ObscCircle(0.7, 0.1, -0.2),
        "annulus": batoid.ObscAnnulus(0.3, 0.9, -0.05, 0.02),
        "rectangle": batoid.ObscRectangle(1.1, 0.4, 0.1, 0.2, 0.3),
        "ray": batoid.ObscRay(0.2, 0.7, -0.1, 0.05),
        "polygon": batoid.ObscPolygon([0.0, 1.0, 0.3, -0.8, -0.4], [-1.0, 0.2, 1.1, 0.6, -0.5]),
        "negation": batoid.ObscNegation(batoid.ObscCircle(0.5)),
        "union": batoid.ObscUnion([batoid.ObscCircle(0.3, 0.5, 0.5), batoid.ObscRectangle(0.5, 2.0),
                                   batoid.ObscRay(0.1, 2.0)]),
        "intersection": batoid.ObscIntersection([batoid.ObscCircle(1.0), batoid.ObscNegation(batoid.ObscCircle(0.4)),
                                                 batoid.ObscRectangle(1.6, 1.2, 0.0, 0.0, -0.2)]),
    }
    out["obsc_pts"] = pts
    for k, o in obscs.items():
        out[f"obsc_{k}"] = np.array([o.contains(a, b) for a, b in zip(pts[0], pts[1])])
    # media
    wl = np.concatenate([np.linspace(300e-9, 1100e-9, 50), W.WAVELENGTHS])
    out["media_wavelengths"] = wl
    out["media_sellmeier"] = silica.getN(wl)
    sumita = batoid.SumitaMedium(2.2705778, -0.010059376, 0.010414999, 0.00028872517, -2.2214495e-05,
                                 1.4258559e-06)
    out["media_sumita"] = sumita.getN(wl)
    air = batoid.Air()
    out["media_air"] = air.getN(wl)
    air2 = batoid.Air(pressure=60.0, temperature=280.0, h2o_pressure=0.5)
    out["media_air2"] = air2.getN(wl)
    tw = np.linspace(320e-9, 1080e-9, 17)
    tn = 1.45 + 0.01 * np.cos(tw * 1e7)
    table = batoid.TableMedium(tw, tn)
    out["media_table_args"] = np.stack([tw, tn])
    out["media_table"] = np.array([table.getN(w) for w in wl])
    return out


def sellmeier_csv_fixture(ref_root):
    """The reference's known-answer vectors for Sellmeier silica
    (tests/test_Medium.py:66-102, testdata/silicaDispersion.csv)."""
    path = os.path.join(ref_root, "tests", "testdata", "silicaDispersion.csv")
    wmicron, ncsv = np.loadtxt(path, delimiter=',').T
    return {"csv_wmicron": wmicron, "csv_n": ncsv}


def _zemax_lsst(path):
    """Hx, Hy, Px, Py and the per-surface rows of a Zemax 'Real Ray Trace
    Data' export (UTF-16), as read by the reference's tests/test_zemax.py:424-428."""
    with open(path, encoding='utf-16-le') as f:
        hp = np.genfromtxt(f, skip_header=13, max_rows=4, usecols=(6,))
    with open(path, encoding='utf-16-le') as f:
        arr = np.genfromtxt(f, skip_header=22, max_rows=18, usecols=list(range(1, 12)))
    return hp, arr


def zemax_fixture(batoid, ref_root):
    """Zemax golden traces of the reference's tests (tests/test_zemax.py:16-63
    HSC at 1e-9, :413-462 LSST at 1e-10) plus the reference's own traces of the
    same rays; optics stored as the parsed YAML configuration."""
    import copy
    import json
    from batoid_gb300.parse import yaml_load
    out = {}
    data = os.path.join(ref_root, "batoid", "data")
    testdata = os.path.join(ref_root, "tests", "testdata")
    # LSST, g band at 500 nm in vacuum
    cfg = yaml_load(open(os.path.join(data, "LSST", "LSST_g_500.yaml")).read())
    out["lsst_config"] = np.array(json.dumps(cfg))
    tel = batoid.parse.parse_optic(copy.deepcopy(cfg["opticalSystem"]))
    for k in range(3):
        hp, arr = _zemax_lsst(os.path.join(testdata, f"LSST_trace_{k}.txt"))
        out[f"lsst{k}_hp"] = hp
        out[f"lsst{k}_zemax"] = arr
        Hx, Hy, Px, Py = hp
        ray = batoid.RayVector.fromStop(Px * 4.18, Py * 4.18, optic=tel, wavelength=500e-9,
                                        theta_x=np.deg2rad(Hx * 1.75), theta_y=np.deg2rad(Hy * 1.75),
                                        projection='zemax')
        out.update(rv_to_dict(ray, f"lsst{k}_in"))
        tf = tel.traceFull(ray)
        out[f"lsst{k}_names"] = np.array(list(tf.keys()))
        for name, v in tf.items():
            r = v["out"].toCoordSys(batoid.CoordSys())
            out.update(rv_to_dict(r, f"lsst{k}_{name}"))
    # HSC (old prescription)
    cfg = yaml_load(open(os.path.join(data, "HSC", "HSC_old.yaml")).read())
    out["hsc_config"] = np.array(json.dumps(cfg))
    tel = batoid.parse.parse_optic(copy.deepcopy(cfg["opticalSystem"]))
    for k in (1, 2, 3):
        with open(os.path.join(testdata, f"HSC_raytrace_{k}.txt")) as f:
            arr = np.loadtxt(f, skiprows=22, usecols=list(range(0, 12)))
        out[f"hsc{k}_zemax"] = arr
        a0 = arr[0]
        rv = batoid.RayVector(a0[1] / 1000, a0[2] / 1000, 16.0, a0[4], a0[5], -a0[6], t=0, wavelength=750e-9)
        tf = tel.traceFull(rv)
        for name, v in tf.items():
            r = v["out"].toCoordSys(batoid.CoordSys())
            out.update(rv_to_dict(r, f"hsc{k}_{name}"))
    return out


def _utf16_rows(path, skip, nrows, cols):
    with open(path, encoding='utf-16-le') as f:
        return np.genfromtxt(f, skip_header=skip, max_rows=nrows, usecols=cols)


def zemax_more_fixture(batoid, ref_root):
    """More Zemax goldens of the reference's tests (tests/test_zemax.py):
    LSST wavefronts (:224-270, 1e-11 m), the HSC Zernike decomposition
    (:189-221), DECam traces and exit pupil (:466-534), CBP traces
    (:536-612) and ComCam traces (:614-700).  Each optic is stored as its
    parsed YAML configuration; the reference's own outputs for the same
    calls are stored beside the Zemax data."""
    import copy
    import json
    from batoid_gb300.parse import yaml_load
    out = {}
    data = os.path.join(ref_root, "batoid", "data")
    testdata = os.path.join(ref_root, "tests", "testdata")

    def load(rel, key):
        cfg = yaml_load(open(os.path.join(data, rel)).read())
        out[f"{key}_config"] = np.array(json.dumps(cfg))
        return batoid.parse.parse_optic(copy.deepcopy(cfg["opticalSystem"]))

    # LSST wavefronts, nx 32, chief reference, zemax projection
    tel = load("LSST/LSST_g_500.yaml", "lsst")
    for k, (thx, thy, fn) in enumerate([(0.0, 0.0, "LSST_wf_0.0_0.0.txt"), (0.0, 1.225, "LSST_wf_0.0_1.225.txt"),
                                        (0.0, 1.75, "LSST_wf_0.0_1.75.txt"),
                                        (1.176, 1.176, "LSST_wf_1.176_1.176.txt")]):
        with open(os.path.join(testdata, fn), encoding='utf-16-le') as f:
            Zwf = np.loadtxt(f, skiprows=16)[::-1]
        out[f"lsstwf{k}_field_deg"] = np.array([thx, thy])
        out[f"lsstwf{k}_zemax"] = Zwf
        bwf = batoid.wavefront(tel, np.deg2rad(thx), np.deg2rad(thy), 500e-9, nx=32, reference='chief',
                               projection='zemax')
        out[f"lsstwf{k}_ref"] = np.asarray(bwf.array.data)
        out[f"lsstwf{k}_ref_mask"] = np.asarray(bwf.array.mask)
    # HSC Zernike decomposition by Zemax: jmax 37 at 0.75 deg, 750 nm, nx 256
    tel = load("HSC/HSC_no_obsc.yaml", "hsc_no_obsc")
    zz = [0.0]
    with open(os.path.join(testdata, "HSC_Zernike.txt")) as f:
        for i, line in enumerate(f):
            if i > 38:
                zz.append(float(line[9:20]))
    out["hsc_zernike_zemax"] = np.array(zz)
    # the reference's wavefront that the reference's zernike fits (GalSim-free part)
    bwf = batoid.wavefront(tel, 0.0, np.deg2rad(0.75), 750e-9, nx=64, reference='chief', projection='zemax')
    out["hsc_wf64_ref"] = np.asarray(bwf.array.data)
    out["hsc_wf64_ref_mask"] = np.asarray(bwf.array.mask)
    # DECam
    tel = load("DECam/DECam.yaml", "decam")
    for k in range(3):
        fn = os.path.join(testdata, f"DECam_raytrace_{k}.txt")
        out[f"decam{k}_hp"] = _utf16_rows(fn, 13, 4, (6,))
        out[f"decam{k}_zemax"] = _utf16_rows(fn, 22, 40, list(range(1, 12)))
        Hx, Hy, Px, Py = out[f"decam{k}_hp"]
        ray = batoid.RayVector.fromStop(Px * 2.005, Py * 2.005, optic=tel, stopSurface=tel['PM'],
                                        wavelength=700e-9, theta_x=np.deg2rad(Hx * 1.1),
                                        theta_y=np.deg2rad(Hy * 1.1), projection='zemax')
        out.update(rv_to_dict(ray, f"decam{k}_in"))
        tf = tel.traceFull(ray)
        out[f"decam{k}_names"] = np.array(list(tf.keys()))
        for name, v in tf.items():
            out.update(rv_to_dict(v["out"].toCoordSys(batoid.CoordSys()), f"decam{k}_{name}"))
    tel.stopSurface = tel['PM']
    out["decam_epp_ref"] = np.asarray(batoid.exitPupilPos(tel, wavelength=700e-9))
    out["decam_D_z"] = np.array(tel['D'].coordSys.origin[2])
    # CBP
    tel = load("LSST/CBP.yaml", "cbp")
    for i in range(1, 5):
        fn = os.path.join(testdata, f"CBP_SRT{i}.txt")
        out[f"cbp{i}_wavelength_um"] = np.atleast_1d(_utf16_rows(fn, 8, 1, (2,)))
        out[f"cbp{i}_hp"] = _utf16_rows(fn, 13, 4, (6,))
        out[f"cbp{i}_rows"] = _utf16_rows(fn, 22, 18, list(range(0, 12)))
    # ComCam, six bands
    for band in "ugrizy":
        load(f"LSST/ComCam_{band}.yaml", f"comcam_{band}")
        for i in (1, 2):
            fn = os.path.join(testdata, f"ComCam_SRT{i}_{band.upper()}.txt")
            out[f"comcam_{band}{i}_wavelength_um"] = np.atleast_1d(_utf16_rows(fn, 8, 1, (2,)))
            out[f"comcam_{band}{i}_hp"] = _utf16_rows(fn, 13, 4, (6,))
            out[f"comcam_{band}{i}_rows"] = _utf16_rows(fn, 22, 18, list(range(0, 12)))
    return out


def wavefront_fixture(batoid):
    """The reference's own batoid.wavefront (batoid/analysis.py:308-388),
    huygensPSF (:181-305) and dkdu (:17-56) on the 12-surface system: three
    fields, an even and an odd pupil grid, both reference points, and both
    lattice paths of huygensPSF (dx given; dx None, from dkdu)."""
    opt = W.tma_optic(batoid, zernike_factory=ref_zernike_factory(batoid))
    A = batoid.analysis
    out = {}
    fields = [(0.0, 0.0), (np.deg2rad(0.8), np.deg2rad(-0.5)), (np.deg2rad(-1.2), np.deg2rad(0.9))]
    out["fields"] = np.array(fields)
    for f, (tx, ty) in enumerate(fields):
        for nx in (32, 33):
            for ref in ("chief", "mean"):
                wf = A.wavefront(opt, tx, ty, 620e-9, nx=nx, reference=ref)
                out[f"wf_{f}_{nx}_{ref}"] = np.asarray(wf.array.data)
                out[f"wf_{f}_{nx}_{ref}_mask"] = np.asarray(wf.array.mask)
                out[f"wf_{f}_{nx}_{ref}_prim"] = np.asarray(wf.primitiveVectors)
        out[f"dkdu_{f}"] = np.asarray(A.dkdu(opt, tx, ty, 620e-9))
    # huygensPSF: field 1 and 2, both lattice paths
    for f in (1, 2):
        tx, ty = fields[f]
        for nx in (32, 33):
            for ref in ("chief", "mean"):
                p = A.huygensPSF(opt, tx, ty, 620e-9, nx=nx, dx=1.5e-6, nxOut=20, reference=ref)
                out[f"hpsf_{f}_{nx}_{ref}_dx"] = np.asarray(p.array)
                out[f"hpsf_{f}_{nx}_{ref}_dx_prim"] = np.asarray(p.primitiveVectors)
        p = A.huygensPSF(opt, tx, ty, 620e-9, nx=24, reference="chief")
        out[f"hpsf_{f}_24_chief_dkdu"] = np.asarray(p.array)
        out[f"hpsf_{f}_24_chief_dkdu_prim"] = np.asarray(p.primitiveVectors)
    return out


def split_fixture(batoid):
    """rSplit on single surfaces (incl. TIR, misses, failed inputs) and
    traceSplit through a two-singlet system with 2 % reflecting coatings."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _split_optic as S
    out = {}
    for c, (surf, m1, m2, coat, cs, speed) in enumerate(S.rsplit_cases(batoid)):
        rv = make_rv(batoid, S.rsplit_rays(speed=speed))
        a, b = batoid.trace.rSplit(surf, rv, m1, m2, coat, coordSys=cs)
        out.update(rv_to_dict(a, f"rs{c}_refr"))
        out.update(rv_to_dict(b, f"rs{c}_refl"))
    for c, (surf, screen, cs) in enumerate(S.screen_cases(batoid)):
        rv = make_rv(batoid, S.rsplit_rays())
        out.update(rv_to_dict(batoid.trace.refractScreen(surf, rv, screen, coordSys=cs), f"scr{c}"))
    out.update(rv_to_dict(S.screen_optic(batoid).trace(make_rv(batoid, S.split_rays())), "scr_optic"))
    optic = S.split_optic(batoid)
    fwd, rev = optic.traceSplit(make_rv(batoid, S.split_rays()), minFlux=1e-4)
    for tag, lst in (("F", fwd), ("R", rev)):
        out[f"{tag}_n"] = np.array(len(lst))
        out[f"{tag}_paths"] = np.array(["|".join(r.path) for r in lst])
        for k, r in enumerate(lst):
            out.update(rv_to_dict(r, f"{tag}{k}"))
    return out


def analysis_fixture(batoid):
    """drdth, dthdr, spot, fftPSF, exitPupilPos and focalLength of the
    12-surface system at one off-axis field (the reference's own analysis
    functions; the GalSim-based ones cannot run here)."""
    opt = W.tma_optic(batoid, zernike_factory=ref_zernike_factory(batoid))
    thx, thy, wl = np.deg2rad(0.6), np.deg2rad(-0.4), 620e-9
    A = batoid.analysis
    out = {"drdth": A.drdth(opt, thx, thy, wl), "dthdr": A.dthdr(opt, thx, thy, wl)}
    sx, sy = A.spot(opt, thx, thy, wl, nx=32)
    out["spot_x"], out["spot_y"] = np.asarray(sx), np.asarray(sy)
    psf = A.fftPSF(opt, thx, thy, wl, nx=32, pad_factor=2)
    out["fft_array"], out["fft_prim"] = np.asarray(psf.array), np.asarray(psf.primitiveVectors)
    out["epp"] = A.exitPupilPos(opt, wl)
    out["focal_length"] = np.array(A.focalLength(opt, thx, thy, wl))
    return out


def factories_fixture(batoid):
    """RayVector.asGrid / asPolar / asSpokes / fromStop of the 12-surface
    system (tests/_factories.py cases), as the reference builds them."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _factories as F
    opt = W.tma_optic(batoid, zernike_factory=ref_zernike_factory(batoid))
    out = {}
    for name, kind, kw in F.cases():
        out.update(rv_to_dict(F.make(batoid, opt, kind, kw), name))
    return out


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref_root = args[0] if args else os.environ.get("BATOID_REF")
    if not ref_root:
        sys.exit("usage: make_golden.py REFERENCE_ROOT [--only-...]  (or set BATOID_REF)")
    os.environ["BATOID_REF"] = ref_root
    batoid = import_reference(ref_root)
    batoid.global_vars._batoid_max_threads = 1
    if "--only-split" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "split.npz"), **split_fixture(batoid))
        return
    if "--only-factories" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "factories.npz"), **factories_fixture(batoid))
        return
    if "--only-zemax-more" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "zemax_more.npz"), **zemax_more_fixture(batoid, ref_root))
        return
    if "--only-wavefront" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "wavefront.npz"), **wavefront_fixture(batoid))
        return
    if "--only-analysis" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "analysis.npz"), **analysis_fixture(batoid))
        return
    np.savez_compressed(os.path.join(HERE, "workloads.npz"), **workload_fixtures(batoid))
    np.savez_compressed(os.path.join(HERE, "primitives.npz"), **primitive_fixtures(batoid))
    np.savez_compressed(os.path.join(HERE, "huygens.npz"), **huygens_fixture(batoid))
    np.savez_compressed(os.path.join(HERE, "sellmeier_csv.npz"), **sellmeier_csv_fixture(ref_root))
    np.savez_compressed(os.path.join(HERE, "zemax.npz"), **zemax_fixture(batoid, ref_root))
    np.savez_compressed(os.path.join(HERE, "split.npz"), **split_fixture(batoid))
    np.savez_compressed(os.path.join(HERE, "analysis.npz"), **analysis_fixture(batoid))
    np.savez_compressed(os.path.join(HERE, "factories.npz"), **factories_fixture(batoid))
    np.savez_compressed(os.path.join(HERE, "zemax_more.npz"), **zemax_more_fixture(batoid, ref_root))
    np.savez_compressed(os.path.join(HERE, "wavefront.npz"), **wavefront_fixture(batoid))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
