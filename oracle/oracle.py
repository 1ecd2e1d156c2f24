"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module, as the checker.  It wraps oracle/liboracle.so (the C restatement in
xct_oracle.c) and, where it was built, oracle/_ref (the reference's own OpenCL kernels
compiled through oracle/ref_shim; see build_ref.py).
"""
import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

ORDER_CANONICAL = 0
ORDER_FWD_LITERAL = 1
ORDER_BP_LITERAL = 2
ORDER_LITERAL = 3
ORDER_GPU = 2


class Geom(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("px", ctypes.c_int), ("pa", ctypes.c_int),
        ("ss", ctypes.c_int), ("depth", ctypes.c_int),
        ("cx", ctypes.c_double),
        ("order", ctypes.c_int), ("fetch_mode", ctypes.c_int),
    ]


def make_geom(nx, ny, px, pa, ss, cx=None, order=ORDER_CANONICAL, fetch_mode=0):
    return Geom(nx, ny, px, pa, ss, max(nx, ny), px * 0.5 if cx is None else float(cx), order, fetch_mode)


def build(force=False):
    """Compile oracle/liboracle.so from xct_oracle.c (no contraction; OpenMP)."""
    src = os.path.join(HERE, "xct_oracle.c")
    deps = [src, os.path.join(HERE, "xct_oracle_body.h"), os.path.join(HERE, "xct_oracle.h")]
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    flags = ["-O2", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # hardware fmaf (same correctly rounded result as a libm call)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.run(["gcc"] + flags + ["-o", tmp, src, "-lm"], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        gp = ctypes.POINTER(Geom)
        for sfx, p, r in (("_f32", fp, ctypes.c_float), ("_f64", dp, ctypes.c_double)):
            getattr(L, "xo_projection" + sfx).argtypes = [p, p, gp, ctypes.c_int, ctypes.c_int, ctypes.c_int, p]
            getattr(L, "xo_osem1" + sfx).argtypes = [p, p, p, gp, ctypes.c_int, ctypes.c_int, p]
            getattr(L, "xo_osem2" + sfx).argtypes = [p, p, p, p, gp, ctypes.c_int]
            getattr(L, "xo_backprojection" + sfx).argtypes = [p, p, gp, ctypes.c_int, p]
            getattr(L, "xo_aart1" + sfx).argtypes = [p, p, p, gp, ctypes.c_int, ctypes.c_int, p]
            getattr(L, "xo_fista_bp" + sfx).argtypes = [p, p, p, p, gp, ctypes.c_int, r, r]
            getattr(L, "xo_bp_fbp" + sfx).argtypes = [p, p, gp, p]
            getattr(L, "xo_sino_correction" + sfx).argtypes = [p, p, fp, gp, ctypes.c_int]
            getattr(L, "xo_adjoint" + sfx).argtypes = [p, p, gp, p]
            getattr(L, "xo_osem_run" + sfx).argtypes = [p, p, p, gp, ip, ctypes.c_int, ctypes.c_int]
        L.xo_power_iteration_f32.argtypes = [fp, gp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp]
        L.xo_fista_run_f32.argtypes = [fp, fp, fp, fp, gp, ctypes.c_int, ip, ctypes.c_int, ctypes.c_float, fp,
                                       ctypes.c_double, ctypes.c_int]
        L.xo_fbp_filter_f32.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp]
        L.xo_fbp_filter_f64.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.xo_base_up_f32.argtypes = [fp, ctypes.c_longlong, ctypes.c_int, fp]
        L.xo_rot_center_shift_f32.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_float, fp]
        L.xo_mask_params_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_float, fp]
        L.xo_set_mask_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, fp]
        L.xo_focus_index.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.xo_focus_index.restype = ctypes.c_double
        L.xo_reslice_f32.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, fp, ctypes.c_float,
                                     ctypes.c_int, fp]
        L.xo_denoise_sinogram_f32.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, fp]
        L.xo_ista3d_f32.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, fp]
        L.xo_fista3d_f32.argtypes = [fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, fp, fp, fp]
        L.xo_trig_f32.argtypes = [fp, ctypes.c_int, fp]
        L.xo_trig_f64.argtypes = [fp, ctypes.c_int, dp]
        L.xo_subset_order.argtypes = [ctypes.c_int, ip]
        _lib = L
    return _lib


def _p(a):
    if a.dtype == np.float32:
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    if a.dtype == np.float64:
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    if a.dtype == np.int32:
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    raise TypeError(a.dtype)


def _sfx(dtype):
    return "_f32" if np.dtype(dtype) == np.float32 else "_f64"


def trig(angles_deg, dtype=np.float32):
    a = np.ascontiguousarray(angles_deg, dtype=np.float32)
    cs = np.empty((a.size, 2), dtype=dtype)
    getattr(lib(), "xo_trig" + _sfx(dtype))(_p(a), a.size, _p(cs))
    return cs


def subset_order(ss):
    out = np.zeros(max(ss, 1), dtype=np.int32)
    lib().xo_subset_order(ss, _p(out))
    return out[:ss]


def projection(img, angles_deg, px, ss=1, sub=0, nrows=None, cx=None, order=ORDER_CANONICAL, dtype=np.float32):
    img = np.ascontiguousarray(img, dtype=dtype)
    ny, nx = img.shape
    pa = len(angles_deg)
    g = make_geom(nx, ny, px, pa, ss, cx, order)
    cs = trig(angles_deg, dtype)
    nrows = pa // ss if nrows is None else nrows
    out = np.zeros((pa, px), dtype=dtype)
    getattr(lib(), "xo_projection" + _sfx(dtype))(_p(img), _p(cs), ctypes.byref(g), sub, ss, nrows, _p(out))
    return out


def osem1(img, meas, angles_deg, ss, sub, nrows=None, cx=None, order=ORDER_CANONICAL, fetch_mode=0,
          dtype=np.float32, ratio=None):
    img = np.ascontiguousarray(img, dtype=dtype)
    meas = np.ascontiguousarray(meas, dtype=dtype)
    ny, nx = img.shape
    pa, px = meas.shape
    g = make_geom(nx, ny, px, pa, ss, cx, order, fetch_mode)
    cs = trig(angles_deg, dtype)
    nrows = pa // ss if nrows is None else nrows
    out = np.zeros((pa, px), dtype=dtype) if ratio is None else ratio
    getattr(lib(), "xo_osem1" + _sfx(dtype))(_p(img), _p(meas), _p(cs), ctypes.byref(g), sub, nrows, _p(out))
    return out


def osem2(img, ratio, angles_deg, ss, sub, cx=None, order=ORDER_CANONICAL, dtype=np.float32):
    img = np.ascontiguousarray(img, dtype=dtype)
    ratio = np.ascontiguousarray(ratio, dtype=dtype)
    ny, nx = img.shape
    pa, px = ratio.shape
    g = make_geom(nx, ny, px, pa, ss, cx, order)
    cs = trig(angles_deg, dtype)
    out = np.empty_like(img)
    getattr(lib(), "xo_osem2" + _sfx(dtype))(_p(img), _p(out), _p(ratio), _p(cs), ctypes.byref(g), sub)
    return out


def backprojection(prj, angles_deg, nx, ny, ss=1, sub=0, order=ORDER_CANONICAL, dtype=np.float32):
    prj = np.ascontiguousarray(prj, dtype=dtype)
    pa, px = prj.shape
    g = make_geom(nx, ny, px, pa, ss, None, order)
    cs = trig(angles_deg, dtype)
    out = np.empty((ny, nx), dtype=dtype)
    getattr(lib(), "xo_backprojection" + _sfx(dtype))(_p(prj), _p(cs), ctypes.byref(g), sub, _p(out))
    return out


def aart1(img, meas, angles_deg, ss, sub, nrows=None, dtype=np.float32):
    img = np.ascontiguousarray(img, dtype=dtype)
    meas = np.ascontiguousarray(meas, dtype=dtype)
    ny, nx = img.shape
    pa, px = meas.shape
    g = make_geom(nx, ny, px, pa, ss, None, ORDER_LITERAL)
    cs = trig(angles_deg, dtype)
    nrows = pa // ss if nrows is None else nrows
    out = np.zeros((pa, px), dtype=dtype)
    getattr(lib(), "xo_aart1" + _sfx(dtype))(_p(img), _p(meas), _p(cs), ctypes.byref(g), sub, nrows, _p(out))
    return out


def fista_bp(img, dprj, angles_deg, ss, sub, alpha, L, dtype=np.float32):
    img = np.ascontiguousarray(img, dtype=dtype)
    dprj = np.ascontiguousarray(dprj, dtype=dtype)
    ny, nx = img.shape
    pa, px = dprj.shape
    g = make_geom(nx, ny, px, pa, ss, None, ORDER_LITERAL)
    cs = trig(angles_deg, dtype)
    out = np.empty_like(img)
    getattr(lib(), "xo_fista_bp" + _sfx(dtype))(_p(img), _p(out), _p(dprj), _p(cs), ctypes.byref(g), sub,
                                                 alpha, L)
    return out


def bp_fbp(fprj, angles_deg, nx, ny, cx=None, dtype=np.float32):
    fprj = np.ascontiguousarray(fprj, dtype=dtype)
    pa, px = fprj.shape
    g = make_geom(nx, ny, px, pa, 1, cx, ORDER_LITERAL)
    cs = trig(angles_deg, dtype)
    out = np.empty((ny, nx), dtype=dtype)
    getattr(lib(), "xo_bp_fbp" + _sfx(dtype))(_p(fprj), _p(cs), ctypes.byref(g), _p(out))
    return out


def default_zp(px):
    """Smallest power of two >= 2*px (4096 for 2048 bins, the reference's default g_zp)."""
    zp = 1
    while zp < 2 * px:
        zp *= 2
    return zp


def fbp_filter(prj, zp=None, dtype=np.float32):
    """Ramp-filtered sinogram of FBP_execution (rows [n][px]); float32 follows FBP.cl
    literally, float64 is the exact-twiddle double transform."""
    prj = np.ascontiguousarray(prj, dtype=dtype)
    shape = prj.shape
    px = shape[-1]
    rows = int(np.prod(shape[:-1]))
    zp = default_zp(px) if zp is None else int(zp)
    out = np.empty_like(prj)
    getattr(lib(), "xo_fbp_filter" + _sfx(dtype))(_p(prj), px, rows, zp, _p(out))
    return out


def fbp(meas, angles_deg, nx, ny, zp=None, cx=None):
    """FBP_execution without sinogram correction: filter, then backProjectionFBP."""
    return bp_fbp(fbp_filter(meas, zp), angles_deg, nx, ny, cx)


def base_up(img, order):
    """Hybrid base-up of one slice; returns (image, slice minimum)."""
    out = np.array(img, dtype=np.float32, copy=True, order="C")
    m = ctypes.c_float(0.0)
    lib().xo_base_up_f32(_p(out), out.size, order, ctypes.byref(m))
    return out, m.value


def shift_values(start, step, n):
    """The shifts start + step*i of rotationCenterSearch_ocl.cpp:140, in float."""
    return [float(np.float32(np.float32(start) + np.float32(step) * np.float32(i))) for i in range(n)]


def rot_center_shift(prj, shift):
    """rotCenterShift (rotCenterSearch.cl:37-49) of one sinogram [pa][px]."""
    prj = np.ascontiguousarray(prj, dtype=np.float32)
    pa, px = prj.shape
    out = np.empty_like(prj)
    lib().xo_rot_center_shift_f32(_p(prj), px, pa, shift, _p(out))
    return out


def mask_params(W, H, shift, ang_min, ang_max):
    prm = np.zeros(13, np.float32)
    lib().xo_mask_params_f32(W, H, shift, ang_min, ang_max, _p(prm))
    return prm


def set_mask(W, H, shift, ang_min, ang_max, w_visit=None):
    """setMask (rotCenterSearch.cl:51-97) for one shift: a [H][W] 0/1 mask."""
    prm = mask_params(W, H, shift, ang_min, ang_max)
    out = np.zeros((H, W), np.float32)
    lib().xo_set_mask_f32(W, H, W if w_visit is None else w_visit, _p(prm), _p(out))
    return out


def focus_index(img, mask, L=0):
    """imgFocusIndex (rotCenterSearch.cl:167-232): literal float order of a work-group of L
    items, or (L = 0) double sums over every pixel."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    H, W = img.shape
    return lib().xo_focus_index(_p(img), _p(mask), W, H, int(L))


def reslice(mt, xshift=None, yshift=None, baseup=0.0, correction=0):
    """reslice (Reslice/reslice.cl:52-71): projections [A][H][W] -> sinograms [H][A][W]."""
    mt = np.ascontiguousarray(mt, dtype=np.float32)
    A, H, W = mt.shape
    xs = None if xshift is None else np.ascontiguousarray(xshift, dtype=np.float32)
    ys = None if yshift is None else np.ascontiguousarray(yshift, dtype=np.float32)
    out = np.empty((H, A, W), np.float32)
    lib().xo_reslice_f32(_p(mt), W, H, A, None if xs is None else _p(xs), None if ys is None else _p(ys),
                         baseup, correction, _p(out))
    return out


def denoise_sinogram(sino, threshold):
    """denoiseSinogram (Reslice/reslice.cl:223-248) on sinograms [H][A][W]."""
    sino = np.ascontiguousarray(sino, dtype=np.float32)
    H, A, W = sino.shape
    out = np.empty_like(sino)
    lib().xo_denoise_sinogram_f32(_p(sino), W, A, H, threshold, _p(out))
    return out


def cs_lambda(cs_lambda_f32):
    """The kernels' float lambda: -D LAMBDA_FISTA is the float CSlambda streamed with six
    significant digits (GPU.cpp:549), parsed as a double literal; lambda =
    LAMBDA_FISTA/L*0.5f with L = 0.5 (FISTA.cl:426, GPU.cpp:343)."""
    d = float("%g" % np.float32(cs_lambda_f32))
    return float(np.float32(d / float(np.float32(0.5)) * 0.5))


def lambda_literal(cs_lambda_f32):
    """The value of -D LAMBDA_FISTA: the float CSlambda streamed with six significant digits
    (GPU.cpp:549, FISTA_programBuild likewise), read back as a double literal."""
    return float("%g" % np.float32(cs_lambda_f32))


def power_iteration(angles_deg, nx, ny, px, ss, trials=30, work_group=1024, fetch_mode=0, layer_mode=0):
    """powerIteration (GPU.cpp:2079-2188): L[ss], the squared norm of (B A) applied to the
    normalised estimate after `trials` rounds, per subset, in the kernels' float order.
    layer_mode 0: powerIter1 projects layer 0 for every subset (its sampling coordinate's
    layer is never set, FISTA.cl:60); 1: each subset's own layer."""
    pa = len(angles_deg)
    g = make_geom(nx, ny, px, pa, ss, None, ORDER_LITERAL, fetch_mode)
    cs = trig(angles_deg, np.float32)
    out = np.zeros(ss, np.float32)
    lib().xo_power_iteration_f32(_p(cs), ctypes.byref(g), trials, work_group, layer_mode, _p(out))
    return out


def fista_run(imgs, meas, angles_deg, ss, it, L, alpha=1.0, cs_lambda_f32=1.0e-4, correction_mode=0,
              sub_order=None, flags=0, order=ORDER_LITERAL):
    """FISTA_execution (GPU.cpp:1755-1924) on a batch meas [dN][pa][px]: the initial image is
    the subset-0 backprojection (imgs only gives the shape), then per subset AART1,
    FISTAbackProjection and ISTA3D (first cycle) / FISTA3D.  flags & 1 stores FISTA3D's
    x_{t+1} as the next image (the reference discards it)."""
    meas = np.ascontiguousarray(meas, dtype=np.float32)
    dN, pa, px = meas.shape
    ny, nx = np.asarray(imgs).shape[-2:]
    g = make_geom(nx, ny, px, pa, ss, None, order)
    cs = trig(angles_deg, np.float32)
    if correction_mode > 0:
        used = np.stack([sino_correction(m, angles_deg, correction_mode) for m in meas])
        res0 = meas.copy()
    else:
        used = meas
        res0 = np.zeros_like(meas)
    so = subset_order(ss) if sub_order is None else np.ascontiguousarray(sub_order, dtype=np.int32)
    out = np.zeros((dN, ny, nx), np.float32)
    Lf = np.ascontiguousarray(L, dtype=np.float32)
    lib().xo_fista_run_f32(_p(out), _p(np.ascontiguousarray(used)), _p(res0), _p(cs), ctypes.byref(g), dN, _p(so),
                           it, float(alpha), _p(Lf), lambda_literal(cs_lambda_f32), int(flags))
    return out


def ista3d(v, lam):
    v = np.ascontiguousarray(v, dtype=np.float32)
    dN, ny, nx = v.shape
    out = np.empty_like(v)
    lib().xo_ista3d_f32(_p(v), nx, ny, dN, lam, _p(out))
    return out


def fista3d(x_in, v, beta, lam):
    x_in = np.ascontiguousarray(x_in, dtype=np.float32)
    v = np.ascontiguousarray(v, dtype=np.float32)
    beta = np.ascontiguousarray(beta, dtype=np.float32)
    dN, ny, nx = v.shape
    w, x, b = np.empty_like(v), np.empty_like(v), np.empty_like(v)
    lib().xo_fista3d_f32(_p(x_in), _p(v), _p(beta), nx, ny, dN, lam, _p(w), _p(x), _p(b))
    return w, x, b


def cs_osem_run(imgs, meas, angles_deg, ss, it, cs_lambda_f32=1.0e-4, sub_order=None, order=ORDER_LITERAL):
    """FISTA_OSEM_execution (GPU.cpp:243-405) on a batch imgs [dN][ny][nx], meas [dN][pa][px]:
    per subset OSEM1 + OSEM2 of every slice, then ISTA3D of the PRE-update image in the first
    cycle (its OS-EM update is discarded, as the reference's kernel arguments have it) and
    FISTA3D(w, v = the OS-EM update, beta) after; the image becomes the proximal result."""
    x = np.array(imgs, dtype=np.float32, copy=True, order="C")
    meas = np.ascontiguousarray(meas, dtype=np.float32)
    dN, ny, nx = x.shape
    so = subset_order(ss) if sub_order is None else np.ascontiguousarray(sub_order, dtype=np.int32)
    lam = cs_lambda(cs_lambda_f32)
    w = x.copy()
    beta = np.zeros_like(x)
    first = True
    for _ in range(it):
        for k in range(ss):
            s = int(so[k])
            v = np.stack([osem2(x[z], osem1(x[z], meas[z], angles_deg, ss, s, order=order), angles_deg, ss, s,
                                order=order) for z in range(dN)])
            if first:
                x = ista3d(x, lam)
                first = False
            else:
                w, x, beta = fista3d(w, v, beta, lam)
    return x


def adjoint(sino, angles_deg, nx, ny, cx=None, dtype=np.float32):
    """Exact adjoint A^T of projection() over all angles."""
    sino = np.ascontiguousarray(sino, dtype=dtype)
    pa, px = sino.shape
    g = make_geom(nx, ny, px, pa, 1, cx, ORDER_CANONICAL)
    cs = trig(angles_deg, dtype)
    out = np.empty((ny, nx), dtype=dtype)
    getattr(lib(), "xo_adjoint" + _sfx(dtype))(_p(sino), _p(cs), ctypes.byref(g), _p(out))
    return out


def sino_correction(meas, angles_deg, mode, dtype=np.float32):
    """sinogramCorrection (reconstShare.cl:35-70), modes 0..4."""
    meas = np.ascontiguousarray(meas, dtype=dtype)
    pa, px = meas.shape
    g = make_geom(px, px, px, pa, 1)
    ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
    out = np.empty_like(meas)
    getattr(lib(), "xo_sino_correction" + _sfx(dtype))(_p(meas), _p(out), _p(ang), ctypes.byref(g), mode)
    return out


def osem_run(img0, meas, angles_deg, ss, it, sub_order=None, cx=None, order=ORDER_CANONICAL, fetch_mode=0,
             cover=False, dtype=np.float32):
    """Full OS-EM of one slice (OSEM_execution's loop); returns the updated image."""
    img = np.array(img0, dtype=dtype, copy=True, order="C")
    meas = np.ascontiguousarray(meas, dtype=dtype)
    ny, nx = img.shape
    pa, px = meas.shape
    g = make_geom(nx, ny, px, pa, ss, cx, order, fetch_mode)
    cs = trig(angles_deg, dtype)
    so = subset_order(ss) if sub_order is None else np.ascontiguousarray(sub_order, dtype=np.int32)
    getattr(lib(), "xo_osem_run" + _sfx(dtype))(_p(img), _p(meas), _p(cs), ctypes.byref(g), _p(so), it,
                                                 1 if cover else 0)
    return img


# ----------------------------------------------------------------------------- oracle/_ref
class RefKernels:
    """The reference's OSEM.cl/reconstShare.cl compiled for one shape (see build_ref.py)."""

    def __init__(self, nx, ny, px, pa, ss, zp=None, cs_lambda="0.0001"):
        import build_ref  # noqa: local module beside this file
        self.shape = (nx, ny, px, pa, ss)
        self.lib = ctypes.CDLL(build_ref.build(nx, ny, px, pa, ss, zp, cs_lambda=cs_lambda))
        self.zp = self.lib.ref_zp_size()
        fp = ctypes.POINTER(ctypes.c_float)
        ip = ctypes.POINTER(ctypes.c_int)
        self.lib.ref_osem_execution.argtypes = [fp, fp, fp, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        self.lib.ref_projection.argtypes = [fp, fp, ctypes.c_int, fp]
        self.lib.ref_backprojection.argtypes = [fp, fp, ctypes.c_int, fp]
        self.lib.ref_sino_correction.argtypes = [fp, fp, ctypes.c_int, fp]
        self.lib.ref_fbp.argtypes = [fp, fp, ctypes.c_int, fp, fp]
        self.lib.ref_bp_fbp.argtypes = [fp, fp, ctypes.c_int, fp]
        self.lib.ref_base_up.argtypes = [fp, ctypes.c_int, ctypes.c_int, fp]
        self.lib.ref_fista_osem_execution.argtypes = [fp, fp, fp, ip, ctypes.c_int, ctypes.c_int]
        self.lib.ref_power_iteration.argtypes = [fp, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int]
        self.lib.ref_fista_execution.argtypes = [fp, fp, fp, ip, ctypes.c_int, ctypes.c_int, ctypes.c_float, fp,
                                                 ctypes.c_int, ctypes.c_int]

    def power_iteration(self, angles_deg, trials=30, work_group=1024, fetch_mode=0):
        ss = self.shape[4]
        out = np.zeros(ss, np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        self.lib.ref_power_iteration(_p(ang), trials, work_group, _p(out), fetch_mode)
        return out

    def fista_execution(self, prjs, angles_deg, sub_order, it, L, alpha=1.0, correction_mode=0, fetch_mode=0):
        nx, ny, px, pa, ss = self.shape
        prjs = np.ascontiguousarray(prjs, dtype=np.float32)
        imgs = np.zeros((prjs.shape[0], ny, nx), np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        so = np.ascontiguousarray(sub_order, dtype=np.int32)
        Lf = np.ascontiguousarray(L, dtype=np.float32)
        self.lib.ref_fista_execution(_p(imgs), _p(prjs), _p(ang), _p(so), prjs.shape[0], it, float(alpha), _p(Lf),
                                     correction_mode, fetch_mode)
        return imgs

    def fista_osem_execution(self, imgs, prjs, angles_deg, sub_order, it):
        imgs = np.array(imgs, dtype=np.float32, copy=True, order="C")
        prjs = np.ascontiguousarray(prjs, dtype=np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        so = np.ascontiguousarray(sub_order, dtype=np.int32)
        self.lib.ref_fista_osem_execution(_p(imgs), _p(prjs), _p(ang), _p(so), imgs.shape[0], it)
        return imgs

    def fbp(self, prjs, angles_deg):
        """FBP_execution: returns (filtered sinograms, images), one per layer."""
        nx, ny, px, pa, ss = self.shape
        prjs = np.ascontiguousarray(prjs, dtype=np.float32)
        dN = prjs.shape[0] if prjs.ndim == 3 else 1
        fprj = np.zeros((dN, pa, px), dtype=np.float32)
        img = np.zeros((dN, ny, nx), dtype=np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        self.lib.ref_fbp(_p(prjs), _p(ang), dN, _p(fprj), _p(img))
        return fprj.reshape(prjs.shape), img.reshape((ny, nx) if prjs.ndim == 2 else (dN, ny, nx))

    def bp_fbp(self, fprj, angles_deg):
        nx, ny, px, pa, ss = self.shape
        out = np.zeros((ny, nx), dtype=np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        self.lib.ref_bp_fbp(_p(np.ascontiguousarray(fprj, dtype=np.float32)), _p(ang), 1, _p(out))
        return out

    def base_up(self, imgs, order):
        """Returns (images after base-up, per-layer minimum)."""
        imgs = np.array(imgs, dtype=np.float32, copy=True, order="C")
        dN = imgs.shape[0] if imgs.ndim == 3 else 1
        mins = np.zeros(dN, dtype=np.float32)
        self.lib.ref_base_up(_p(imgs), dN, order, _p(mins))
        return imgs, mins

    def osem_execution(self, imgs, prjs, angles_deg, sub_order, it, fetch_mode=0):
        imgs = np.array(imgs, dtype=np.float32, copy=True, order="C")
        prjs = np.ascontiguousarray(prjs, dtype=np.float32)
        dN = imgs.shape[0] if imgs.ndim == 3 else 1
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        so = np.ascontiguousarray(sub_order, dtype=np.int32)
        self.lib.ref_osem_execution(_p(imgs), _p(prjs), _p(ang), _p(so), dN, it, fetch_mode)
        return imgs

    def projection(self, img, angles_deg, sub=0):
        nx, ny, px, pa, ss = self.shape
        out = np.zeros((pa, px), dtype=np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        self.lib.ref_projection(_p(np.ascontiguousarray(img, dtype=np.float32)), _p(ang), sub, _p(out))
        return out

    def sino_correction(self, prj, angles_deg, mode):
        nx, ny, px, pa, ss = self.shape
        out = np.zeros((pa, px), dtype=np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        self.lib.ref_sino_correction(_p(np.ascontiguousarray(prj, dtype=np.float32)), _p(ang), mode, _p(out))
        return out

    def backprojection(self, prj, angles_deg, sub=0):
        nx, ny, px, pa, ss = self.shape
        out = np.zeros((ny, nx), dtype=np.float32)
        ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
        self.lib.ref_backprojection(_p(np.ascontiguousarray(prj, dtype=np.float32)), _p(ang), sub, _p(out))
        return out


class RefRotCenter:
    """The reference's rotCenterSearch.cl compiled for one image size (build_ref.build_rcs)."""

    def __init__(self, width, height):
        import build_ref  # noqa: local module beside this file
        self.shape = (width, height)
        self.lib = ctypes.CDLL(build_ref.build_rcs(width, height))
        fp = ctypes.POINTER(ctypes.c_float)
        c_i, c_f = ctypes.c_int, ctypes.c_float
        self.lib.rcs_rot_center_shift.argtypes = [fp, c_i, c_i, c_i, c_f, c_f, fp]
        self.lib.rcs_focus_index.argtypes = [fp, c_i, c_i, c_i, c_f, c_f, c_f, c_f, fp, fp]

    def rot_center_shift(self, prj, n, start, step):
        prj = np.ascontiguousarray(prj, dtype=np.float32)
        pa, px = prj.shape
        out = np.zeros((n, pa, px), np.float32)
        self.lib.rcs_rot_center_shift(_p(prj), px, pa, n, start, step, _p(out))
        return out

    def focus_index(self, imgs, L, start, step, ang_ini, ang_fin, offsetN=0):
        """Returns (masks [n][H][W], findex [n])."""
        imgs = np.ascontiguousarray(imgs, dtype=np.float32)
        n = imgs.shape[0]
        W, H = self.shape
        masks = np.zeros((n, H, W), np.float32)
        fi = np.zeros(n, np.float32)
        self.lib.rcs_focus_index(_p(imgs), n, L, offsetN, start, step, ang_ini, ang_fin, _p(masks), _p(fi))
        return masks, fi


class RefReslice:
    """The reference's reslice.cl compiled for one (width, height, angles) (build_reslice)."""

    def __init__(self, width, height, n_angles):
        import build_ref  # noqa: local module beside this file
        self.shape = (width, height, n_angles)
        self.lib = ctypes.CDLL(build_ref.build_reslice(width, height, n_angles))
        fp = ctypes.POINTER(ctypes.c_float)
        self.lib.ref_reslice.argtypes = [fp, fp, fp, ctypes.c_float, ctypes.c_int, fp]
        self.lib.ref_denoise.argtypes = [fp, ctypes.c_float, fp]

    def reslice(self, mt, xshift=None, yshift=None, baseup=0.0, correction=0):
        W, H, A = self.shape
        xs = np.zeros(A, np.float32) if xshift is None else np.ascontiguousarray(xshift, dtype=np.float32)
        ys = np.zeros(A, np.float32) if yshift is None else np.ascontiguousarray(yshift, dtype=np.float32)
        out = np.zeros((H, A, W), np.float32)
        self.lib.ref_reslice(_p(np.ascontiguousarray(mt, dtype=np.float32)), _p(xs), _p(ys), baseup, correction,
                             _p(out))
        return out

    def denoise(self, sino, threshold):
        out = np.zeros_like(sino, dtype=np.float32)
        self.lib.ref_denoise(_p(np.ascontiguousarray(sino, dtype=np.float32)), threshold, _p(out))
        return out


def reslice_available():
    import build_ref
    return build_ref.reslice_available()


def rcs_available():
    import build_ref
    return build_ref.rcs_available()


def ref_available():
    import build_ref
    return build_ref.available()
