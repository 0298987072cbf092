"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout where the reference tree is available ($DEFORMETRICA_REFERENCE_DIR, else the
default location oracle.reference_root() names):

    python tests/golden/make_golden.py [REFERENCE_ROOT]

It builds oracle/_ref (the reference's own ExactKernel / AbstractKernel compiled from its
sources by oracle/build_ref.sh) and records its outputs:

* ``kernel_precision.npz`` -- every ExactKernel method on the fixture of the reference's kernel
  tests (tests/unit_tests/kernels/AbstractTestKernelPrecision.{h,cxx}: sigma = 1.88, X 501 rows,
  Y 201 rows, entries exp(-U) with std::mt19937(1) re-seeded for every matrix), i.e. the
  operations TestKernelPrecisionCUDA.cxx:17-203 compares, plus the remaining overloads.
* ``kernel_random.npz`` -- the same methods on seeded, non-degenerate inputs (sigma 0.2 and 0.05,
  uniform points, N(0,1) weights, ragged sizes).
* ``parallel_transport.npz`` -- the inputs and ground truth of
  tests/unit_tests/parallel-transport/TestParallelTransport.cxx:19-85 (read from the reference's
  DLM text files), which pin the shooting oracle (oracle/deformation.py).
* ``skull_registration.npz`` -- functional test 5 (registration/landmark/2d/skulls: a 2-D
  NonOrientedPolyline registration): the two polylines (x, y of the VTK points, 2-point LINES
  cells), the initial control points and the final FastGradientAscent state.
* ``p3m_reference.npz`` -- every method of the reference's P3MKernel<double, d>
  (src/support/kernels/P3MKernel.cxx) on seeded 2-D and 3-D cases (32^d and 64^d grids, one with
  points outside the data domain), compiled from the reference's source against the ITK stand-ins
  of oracle/ref_shim (direct discrete Fourier transforms in place of VNL's FFT).
* ``amygdala_registration.npz`` -- functional test 6 of the reference
  (tests/functional_tests/configure.ini [Test6], registration/landmark/3d/amygdalas): the two
  meshes as the reference reads them (VTK float points, triangles re-oriented by its normals
  filter), the initial control points, and the final FastGradientAscent state the reference
  stored in deformetrica-state.bin (decoded by deformetrica_code_gb300.formats).

The fixtures are small (tens to hundreds of KB) and are committed; the GPU machine never needs the
reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from tests.golden.fixtures import precision_fixture, random_cases  # noqa: E402


def read_dlm(path: str) -> np.ndarray:
    """readMatrixDLM (src/io/MatrixDLM.cxx): whitespace-separated rows, one matrix."""
    rows = [ln.split() for ln in open(path).read().strip().splitlines() if ln.strip()]
    return np.array([[float(v) for v in r] for r in rows])


def read_multiple_dlm(path: str) -> list[np.ndarray]:
    """readMultipleMatrixDLM: a header 'count rows cols', then each matrix after a blank line."""
    toks = open(path).read().split()
    cnt, r, c = int(toks[0]), int(toks[1]), int(toks[2])
    vals = np.array([float(t) for t in toks[3:]])
    return [vals[k * r * c:(k + 1) * r * c].reshape(r, c) for k in range(cnt)]


def all_ops(lib, X, Y, W, Z, sigma, W3):
    """Every ExactKernel method of the reference on one input set (keys name the method)."""
    d = X.shape[1]
    out = {}
    out["convolve"] = lib.convolve(X, Y, W, sigma)
    out["grad_varlin"] = lib.grad_varlin(X, Y, W, sigma)
    Za = Z[:, :W.shape[1]] if Z.shape[1] >= W.shape[1] else np.tile(Z, (1, 3))[:, :W.shape[1]]
    out["grad_alpha_alpha"] = Za
    out["grad_alpha"] = lib.grad_alpha(X, Y, W, sigma, Za)
    for dim in range(d):
        out[f"grad_dim_{dim}"] = lib.grad_dim(Y, Y, W, sigma, dim)  # TestKernelPrecisionCUDA uses Y
        out[f"grad_dim_x_{dim}"] = lib.grad_dim(X, Y, W, sigma, dim)
    if X.shape[0] >= Y.shape[0]:
        out["grad_kdp"] = lib.grad_kdp(X, Y, W, sigma, W.shape[1] - 1, d - 1)
    else:  # the reference's bounds-checked row access throws (ExactKernel.cxx:343-347)
        try:
            lib.grad_kdp(X, Y, W, sigma, W.shape[1] - 1, d - 1)
            raise AssertionError("reference accepted ConvolveGradient(X,k,dp) with nx < ny")
        except oracle.kernels.OracleError:
            out["grad_kdp_raises"] = np.array(1)
    out["hess_full"] = lib.hess_full(X, Y, W, sigma)
    for r in range(d):
        for c in range(d):
            out[f"hess_rowcol_{r}{c}"] = lib.hess_rowcol(X, Y, W, sigma, r, c)
    out["hess_kdpdq"] = lib.hess_kdpdq(X, Y, W, sigma, 0, 0, d - 1)
    out["special_hessian"] = lib.special_hessian(Y, W3, sigma, W3)
    return out


def main(ref_root: str | None = None):
    ref_root = ref_root or oracle.reference_root()
    if oracle.build_reference(ref_root) is None:
        raise SystemExit(f"reference tree not found at {ref_root}")
    ref = oracle.load("reference")
    port = oracle.load("port")

    # 1. the reference's own kernel-test fixture
    fx = precision_fixture()
    res = {}
    for d in (2, 3):
        X, Y, Z = fx[f"X{d}D"], fx[f"Y{d}D"], fx[f"Z{d}D"]
        W3 = fx[f"W{d}D"]
        for wname in ([f"W{d}D", "W4D"] if d == 2 else [f"W{d}D", "W6D"]):
            W = fx[wname]
            for k, v in all_ops(ref, X, Y, W, Z, fx["kernel_width"], W3).items():
                res[f"d{d}_{wname}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "kernel_precision.npz"), **res)

    # 2. non-degenerate seeded cases
    res = {}
    for name, case in random_cases().items():
        for k, v in all_ops(ref, case["X"], case["Y"], case["W"], case["Z"], case["sigma"],
                            case["W3"]).items():
            res[f"{name}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "kernel_random.npz"), **res)

    del port

    # 3. parallel-transport unit-test data (TestParallelTransport.cxx:19-85)
    pt = os.path.join(ref_root or oracle.reference_root(), "tests", "unit_tests", "parallel-transport", "data")
    np.savez_compressed(
        os.path.join(HERE, "parallel_transport.npz"),
        cp_regression=read_dlm(os.path.join(pt, "CPRegression.txt")),
        mom_regression=read_dlm(os.path.join(pt, "MomRegression.txt")),
        cp_transport=read_dlm(os.path.join(pt, "CPToTransport.txt")),
        mom_transport=read_multiple_dlm(os.path.join(pt, "MomToTransport.txt"))[0],
        ground_truth_mom=read_dlm(os.path.join(pt, "GroundTruthMom.txt")),
        kernel_width=np.array(15.0),
        number_of_time_points=np.array(30),
    )
    # 4. functional tests 5 and 6: landmark registrations of two skull curves, two amygdala meshes
    skull_fixture(ref_root)
    amygdala_fixture(ref_root)
    # 5. volume-mesh gradient unit test and the point-cloud example's point sets
    volume_fixture(ref_root)
    # 6. functional test 8: a two-object curve atlas of three subjects
    parabola_fixture(ref_root)
    # 7. functional test 7: a geodesic regression of three skull curves
    regression_fixture(ref_root)
    # 8. functional test 2: a banana surface atlas estimated by GradientAscent
    banana_fixture(ref_root)
    # 9. the image-grid methods of ExactKernel through the ITK stand-ins of oracle/ref_shim
    image_fixture(ref_root)
    # 10. every P3MKernel method through the same stand-ins (direct DFTs in place of VNL's FFT)
    p3m_fixture(ref_root)
    print("wrote", sorted(os.listdir(HERE)))


def _formats():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "formats", os.path.join(os.path.dirname(os.path.dirname(HERE)), "deformetrica_code_gb300", "formats.py"))
    F = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(F)
    return F


def skull_fixture(ref_root: str | None = None):
    """Inputs and expected final state of the reference's skull registration (model.xml:
    NonOrientedPolyline, data-sigma 1, object kernel width 40, deformation kernel width 60, 6 time
    points; optimization_parameters.xml: FastGradientAscent, 10 iterations, default initial step
    1e-3 (SparseDiffeoParameters.cxx:82))."""
    F = _formats()
    from oracle.optimize import initial_control_points
    d = os.path.join(ref_root or oracle.reference_root(), "tests", "functional_tests", "registration", "landmark", "2d", "skulls")
    tp, tf = F.read_vtk_polydata(os.path.join(d, "data", "template.vtk"))
    gp, gf = F.read_vtk_polydata(os.path.join(d, "data", "skull_sapiens.vtk"))
    tp, gp = np.ascontiguousarray(tp[:, :2]), np.ascontiguousarray(gp[:, :2])  # a 2-D object
    st = F.read_deformation_state(os.path.join(d, "deformetrica-state.bin"))
    cp0 = initial_control_points(tp[tf].mean(axis=1), 60.0)  # the segment centres' box
    np.savez_compressed(
        os.path.join(HERE, "skull_registration.npz"),
        tmpl_pts=tp, tmpl_segs=tf, tgt_pts=gp, tgt_segs=gf, cp0=cp0,
        kernel_width=np.array(60.0), data_kernel_width=np.array(40.0), data_sigma2=np.array(1.0),
        number_of_time_points=np.array(6), initial_step=np.array(1e-3), max_iterations=np.array(10),
        **{f"state_{k}": np.asarray(v) for k, v in st.items()})


def amygdala_fixture(ref_root: str | None = None):
    """Inputs and expected final state of the reference's amygdala registration (model.xml:
    OrientedSurfaceMesh, data-sigma 0.1, object and deformation kernel width 10, 10 time points;
    optimization_parameters.xml: FastGradientAscent, initial step 1e-7, 10 iterations)."""
    F = _formats()
    from oracle.optimize import initial_control_points
    d = os.path.join(ref_root or oracle.reference_root(), "tests", "functional_tests", "registration", "landmark", "3d", "amygdalas")
    tp, tf_raw = F.read_vtk_polydata(os.path.join(d, "data", "decimatedAmygdala1.vtk"))
    gp, gf_raw = F.read_vtk_polydata(os.path.join(d, "data", "decimatedAmygdala2.vtk"))
    tf, gf = F.reorient_like_reader(tp, tf_raw), F.reorient_like_reader(gp, gf_raw)
    st = F.read_deformation_state(os.path.join(d, "deformetrica-state.bin"))
    cp0 = initial_control_points(tp[tf].mean(axis=1), 10.0)  # the template's triangle centres' box
    np.savez_compressed(
        os.path.join(HERE, "amygdala_registration.npz"),
        tmpl_pts=tp, tmpl_tris_raw=tf_raw, tmpl_tris=tf, tgt_pts=gp, tgt_tris_raw=gf_raw, tgt_tris=gf, cp0=cp0,
        kernel_width=np.array(10.0), data_kernel_width=np.array(10.0), data_sigma2=np.array(0.01),
        number_of_time_points=np.array(10), initial_step=np.array(1e-7), max_iterations=np.array(10),
        **{f"state_{k}": np.asarray(v) for k, v in st.items()})


def volume_fixture(ref_root: str | None = None):
    """Meshes of the reference's volume-gradient unit test (TestVolumeGradient.cxx:86-120: kernel
    width 1, forward differences of step 1e-5f, |analytic - numeric| <= 1e-5): a tetrahedral cube
    deformed towards a ball in 3-D, a triangulated square towards a disk in 2-D (the 2-D objects keep
    the first two coordinates), and the two 4-point sets of the 2-D point-cloud example."""
    F = _formats()
    g = os.path.join(ref_root or oracle.reference_root(), "tests", "unit_tests", "geometries", "data")
    out = {}
    for name, dim in (("VolumeCube", 3), ("VolumeBall", 3), ("VolumeSquare", 2), ("VolumeDisk", 2)):
        p, c = F.read_vtk_polydata(os.path.join(g, name + ".vtk"))
        out[f"{name}_pts"] = np.ascontiguousarray(p[:, :dim])
        out[f"{name}_cells"] = np.asarray(c, dtype=np.int32)
    e = os.path.join(ref_root or oracle.reference_root(), "examples", "registration", "landmark", "2d", "simple_point_cloud", "data")
    for name in ("sourcePoints", "targetPoints"):
        p, _ = F.read_vtk_polydata(os.path.join(e, name + ".vtk"))
        out[f"{name}_pts"] = np.ascontiguousarray(p[:, :2])
    np.savez_compressed(os.path.join(HERE, "volume_meshes.npz"), kernel_width=np.array(1.0),
                        fd_step=np.array(float(np.float32(1e-5))), tolerance=np.array(1e-5), **out)


def parabola_fixture(ref_root: str | None = None):
    """Inputs and expected final state of the reference's parabola atlas (functional test 8,
    model.xml: DeterministicAtlas, two OrientedPolyline objects "line" and "wave", object kernel
    width 0.2, data-sigma 1, deformation kernel width 0.2, 10 time points; three subjects;
    optimization_parameters.xml: FastGradientAscent (the default), initial step 1e-3,
    10 iterations, 10 line-search iterations. Its smoothing-kernel-width-ratio element is not a key
    the reference's XML converter reads (it reads smoothing-kernel-with-ratio,
    XmlConfigurationConverter.cxx:228), so the ratio keeps its default 1: smoothing width 0.2)."""
    F = _formats()
    from oracle.optimize import initial_control_points
    d = os.path.join(ref_root or oracle.reference_root(), "tests", "functional_tests", "atlas", "landmark", "2d", "parabola")
    out = {}
    centres = []
    for i in (1, 2):
        p, c = F.read_vtk_polydata(os.path.join(d, "data", f"{i}-meantemplate.vtk"))
        out[f"tmpl{i}_pts"], out[f"tmpl{i}_segs"] = np.ascontiguousarray(p[:, :2]), c
        centres.append(p[c].mean(axis=1)[:, :2])
        for s in (1, 2, 3):
            q, e = F.read_vtk_polydata(os.path.join(d, "data", f"{i}-subject{s}.vtk"))
            out[f"subj{s}_obj{i}_pts"], out[f"subj{s}_obj{i}_segs"] = np.ascontiguousarray(q[:, :2]), e
    st = F.read_deformation_state(os.path.join(d, "deformetrica-state.bin"))
    for k in ("template", "aux_template", "grad_template"):
        st[k] = np.concatenate(st[k])
    np.savez_compressed(
        os.path.join(HERE, "parabola_atlas.npz"), cp0=initial_control_points(np.concatenate(centres), 0.2),
        kernel_width=np.array(0.2), data_kernel_width=np.array(0.2), data_sigma2=np.array(1.0),
        smoothing_width=np.array(0.2), number_of_time_points=np.array(10), initial_step=np.array(1e-3),
        max_iterations=np.array(10), **out, **{f"state_{k}": np.asarray(v) for k, v in st.items()})


def regression_fixture(ref_root: str | None = None):
    """Inputs and expected final state of the reference's geodesic regression (functional test 7,
    model.xml: Regression, initial CP spacing 40, one NonOrientedPolyline object with data kernel
    width 40 and data-sigma 1, deformation kernel width 60, 5 time points from t0 = 0 to tn = 5;
    data_set.xml: observations at ages 0, 3, 5, i.e. time indices int((age - t0)(T - 1)/(tn - t0)
    + 0.5) = 0, 2, 4 (estimate_geodesic_regression.cxx:229-237); optimization_parameters.xml:
    FastGradientAscent, 10 iterations, tolerance 1e-3, default initial step 1e-3; smoothing width
    1 x 60, the default ratio). The state's fixed effects are ControlPoints, InitialMomenta and
    TemplateData (fixed, extrapolated, gradient)."""
    F = _formats()
    from oracle.optimize import initial_control_points
    d = os.path.join(ref_root or oracle.reference_root(), "tests", "functional_tests", "regression", "landmark", "2d", "skulls")
    tp, tc = F.read_vtk_polydata(os.path.join(d, "data", "template.vtk"))
    out = {"tmpl_pts": np.ascontiguousarray(tp[:, :2]), "tmpl_segs": tc}
    for k, name in enumerate(("skull_australopithecus", "skull_habilis", "skull_sapiens")):
        p, c = F.read_vtk_polydata(os.path.join(d, "data", name + ".vtk"))
        out[f"obs{k}_pts"], out[f"obs{k}_segs"] = np.ascontiguousarray(p[:, :2]), c
    blobs, head = F.read_state_blobs(os.path.join(d, "deformetrica-state.bin"))
    named = [b for b in blobs if b["name"] is not None]
    vecs = [b for b in blobs if b["name"] is None]
    st = {"step": vecs[0]["value"], "grad_sq_norms": vecs[1]["value"],
          "history": np.stack([b["value"] for b in vecs[2:]])}
    for i, what in enumerate(("", "aux_", "grad_")):
        for j, key in enumerate(("control_points", "momenta", "template")):
            assert named[3 * i + j]["name"] == ("ControlPoints", "InitialMomenta", "TemplateData")[j]
            st[what + key] = named[3 * i + j]["value"]
    tau_i = next(i for i, t in enumerate(head) if "." in t)
    uints = [int(t) for t in head[:tau_i] if t.isdigit()]
    st["tau"], st["iter"], st["freeze_counter"] = float(head[tau_i]), uints[-6], uints[-5]
    np.savez_compressed(
        os.path.join(HERE, "regression_skulls.npz"), cp0=initial_control_points(tp[tc].mean(axis=1)[:, :2], 40.0),
        times=np.array([0, 2, 4]), t0=np.array(0.0), tn=np.array(5.0), number_of_time_points=np.array(5),
        kernel_width=np.array(60.0), data_kernel_width=np.array(40.0), data_sigma2=np.array(1.0),
        smoothing_width=np.array(60.0), initial_step=np.array(1e-3), max_iterations=np.array(10),
        tolerance=np.array(1e-3), **out, **{f"state_{k}": np.asarray(v) for k, v in st.items()})


def banana_fixture(ref_root: str | None = None):
    """Inputs and expected final state of the reference's banana atlas (functional test 2,
    model.xml: DeterministicAtlas, OrientedSurfaceMesh with data kernel width 0.5 and data-sigma
    0.5, re-oriented normals, initial CP spacing 0.3, deformation kernel width 1, 20 time points;
    three subjects; optimization_parameters.xml: GradientAscent, 150 iterations, 20 line-search
    iterations, step expand 2; default initial step 1e-3, shrink 0.5, tolerance 1e-4, smoothing
    ratio 1). GradientAscent stores the step, the history, the fixed effects (ControlPoints,
    TemplateData), the momenta and the gradients at the final point (GradientAscent.cxx:226-236)."""
    F = _formats()
    from oracle.optimize import initial_control_points
    d = os.path.join(ref_root or oracle.reference_root(), "tests", "functional_tests", "atlas", "landmark", "3d", "banana")
    tp, tf_raw = F.read_vtk_polydata(os.path.join(d, "data", "template.vtk"))
    tf = F.reorient_like_reader(tp, tf_raw)
    out = {"tmpl_pts": tp, "tmpl_tris": tf}
    for i in (1, 2, 3):
        p, f = F.read_vtk_polydata(os.path.join(d, "data", f"banana_{i}.vtk"))
        out[f"subj{i}_pts"], out[f"subj{i}_tris"] = p, F.reorient_like_reader(p, f)
    blobs, head = F.read_state_blobs(os.path.join(d, "deformetrica-state.bin"))
    vecs = [b["value"] for b in blobs if b["name"] is None]
    named = [b for b in blobs if b["name"] is not None]
    cps = [b["value"] for b in named if b["name"] == "ControlPoints"]
    tds = [b["value"] for b in named if b["name"] == "TemplateData"]
    moms = [b["value"] for b in named if b["name"] == "Momenta"]
    st = {"step": vecs[0], "history": np.stack(vecs[1:]), "control_points": cps[0], "grad_control_points": cps[1],
          "template": tds[0], "grad_template": tds[1], "momenta": np.stack(moms[:3]),
          "grad_momenta": np.stack(moms[3:6]), "iter": [int(t) for t in head if t.isdigit()][-16]}
    np.savez_compressed(
        os.path.join(HERE, "banana_atlas.npz"), cp0=initial_control_points(tp[tf].mean(axis=1), 0.3),
        kernel_width=np.array(1.0), data_kernel_width=np.array(0.5), data_sigma2=np.array(0.25),
        smoothing_width=np.array(1.0), number_of_time_points=np.array(20), initial_step=np.array(1e-3),
        max_iterations=np.array(150), max_line_search=np.array(20), expand=np.array(2.0), **out,
        **{f"state_{k}": np.asarray(v) for k, v in st.items()})




def image_cases():
    """Seeded image-grid cases (deformed image points, control points over the image and past its
    edges so windows are cropped, dv = d and dv = 4 weights): name -> arrays."""
    rng = np.random.default_rng(11)
    cases = {}
    for name, size, origin, spacing, sigma, ny, dv in (
            ("d2", [23, 17], [0.5, -1.0], [1.0, 1.5], 2.2, 11, 2),
            ("d2w4", [16, 21], [-2.0, 0.25], [0.75, 1.0], 1.7, 9, 4),
            ("d3", [11, 9, 8], [0.0, 0.5, -0.5], [1.0, 1.2, 0.8], 1.45, 10, 3),
            ("d3w4", [9, 10, 7], [1.0, -1.0, 0.0], [1.1, 0.9, 1.0], 1.2, 8, 4)):
        d = len(size)
        from oracle import image as im
        n = int(np.prod(size))
        x = im.image_points(origin, spacing, size) + 0.15 * rng.standard_normal((n, d))
        lo = np.asarray(origin)
        hi = lo + np.asarray(spacing) * (np.asarray(size) - 1)
        y = rng.uniform(lo - 1.5, hi + 1.5, (ny, d))
        cases[name] = dict(x=x, y=y, w=rng.standard_normal((ny, dv)), alpha=rng.standard_normal((n, dv)),
                           sigma=np.array(sigma), origin=np.asarray(origin, float),
                           spacing=np.asarray(spacing, float), size=np.asarray(size, np.int64))
    return cases


def image_fixture(ref_root: str | None = None):
    """ExactKernel::ConvolveImageFast (dv = d cases) and both ConvolveGradientImageFast overloads
    (ExactKernel.cxx:76-129, 207-290), computed by the reference's own compiled code on the ITK
    stand-ins of oracle/ref_shim: tests/golden/image_fast.npz."""
    oracle.build_reference(ref_root)
    ref = oracle.load("reference")
    res = {}
    for name, c in image_cases().items():
        for k, v in c.items():
            res[f"{name}_{k}"] = v
        args = (c["x"], c["y"], c["w"], float(c["sigma"]), c["origin"], c["spacing"], c["size"])
        if c["w"].shape[1] == c["x"].shape[1]:
            res[f"{name}_convolve"] = ref.image_fast(0, *args)
        res[f"{name}_gradient"] = ref.image_fast(1, *args)
        res[f"{name}_gradient_alpha"] = ref.image_fast(2, *args, alpha=c["alpha"])
    np.savez_compressed(os.path.join(HERE, "image_fast.npz"), **res)


def p3m_cases():
    """Seeded P3M cases: name -> arrays (targets x, sources y, weights w, alpha, the special
    Hessian's sources / momenta / xi, the data domain lo/hi, sigma, spacing ratio, padding)."""
    rng = np.random.default_rng(17)
    cases = {}
    for name, d, nx, ny, dv, sigma, ratio, padding, span, dom in (
            ("d2", 2, 160, 190, 2, 0.2, 0.2, 3.0, (0.0, 1.0), None),
            ("d2out", 2, 150, 170, 3, 0.1, 0.2, 3.0, (-0.5, 1.5), (0.2, 0.8)),
            ("d3", 3, 90, 110, 3, 0.3, 0.5, 3.0, (0.0, 1.0), None),
            ("d3dv2", 3, 80, 100, 2, 0.25, 0.4, 2.0, (0.0, 1.0), None)):
        x, y = rng.uniform(*span, (nx, d)), rng.uniform(*span, (ny, d))
        if dom is None:
            both = np.concatenate([x, y])
            lo, hi = both.min(axis=0), both.max(axis=0)
        else:
            lo, hi = np.full(d, dom[0]), np.full(d, dom[1])
        ys = rng.uniform(*span, (ny, d))
        cases[name] = dict(x=x, y=y, w=rng.standard_normal((ny, dv)), alpha=rng.standard_normal((nx, dv)),
                           ys=ys, beta=rng.standard_normal((ny, d)), xi=rng.standard_normal((ny, d)),
                           lo=lo, hi=hi, ys_lo=ys.min(axis=0), ys_hi=ys.max(axis=0), sigma=np.array(sigma),
                           ratio=np.array(ratio), padding=np.array(padding))
    return cases


def p3m_fixture(ref_root: str | None = None):
    """Every P3MKernel method (P3MKernel.cxx:1245-1729, and AbstractKernel::ConvolveSpecialHessian over
    its Hessians) computed by the reference's own compiled code: tests/golden/p3m_reference.npz."""
    oracle.build_reference(ref_root)
    ref = oracle.load("reference")
    res = {}
    for name, c in p3m_cases().items():
        for k, v in c.items():
            res[f"{name}_{k}"] = v
        d = c["x"].shape[1]
        common = dict(lo=c["lo"], hi=c["hi"], ratio=float(c["ratio"]), padding=float(c["padding"]))
        xyws = (c["x"], c["y"], c["w"], float(c["sigma"]))
        res[f"{name}_convolve"] = ref.p3m("convolve", *xyws, **common)
        res[f"{name}_gradient"] = ref.p3m("gradient", *xyws, **common)
        res[f"{name}_gradient_alpha"] = ref.p3m("gradient_alpha", *xyws, alpha=c["alpha"], **common)
        res[f"{name}_gradient_dim"] = ref.p3m("gradient_dim", *xyws, args=(d - 1,), **common)
        res[f"{name}_hessian"] = ref.p3m("hessian", *xyws, **common)
        res[f"{name}_hessian_rowcol"] = ref.p3m("hessian_rowcol", *xyws, args=(d - 1, 0), **common)
        res[f"{name}_special_hessian"] = ref.p3m(
            "special_hessian", c["ys"], c["ys"], c["beta"], float(c["sigma"]), c["ys_lo"], c["ys_hi"],
            float(c["ratio"]), float(c["padding"]), alpha=c["xi"])
    np.savez_compressed(os.path.join(HERE, "p3m_reference.npz"), **res)


if __name__ == "__main__":
    main(*(sys.argv[1:2]))
