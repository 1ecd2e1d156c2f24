"""Python front end of libxct, the GB300 OS-EM library (ctypes over include/xct.h).

The product is the C ABI in ``libxct.so``; this module loads it and mirrors the
reference's host interface for the OS-EM path of CT_reconstruction
(CT_reconstruction/CT_reconstruction.hpp:68-90, GPU.cpp:125-663):

* ``Context``      -- replaces OCL_platform_device (one CUDA device);
* ``OSEMPlan``     -- replaces OSEM_programBuild + the image objects of OSEM_execution;
* ``OSEM_execution(plan, sub, reconst_img, prj_img, dN, it, prjCorrection)`` -- the
  reference's executor on device tensors, same argument meaning;
* ``OSEM_thread(plan, sub, imgs, prjs, startN, endN, it)`` -- host arrays in, results
  written back into ``imgs`` (the reference's host<->device staging, GPU.cpp:408-476).

Errors raise ``XCTError`` carrying the library's status code and message (the reference
prints and exits, GPU.cpp:231-237; callers that want that behaviour catch and exit).
There is no CPU fallback: if the CUDA library is missing, importing works but every
call raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libxct.so")

XCT_OK = 0
XCT_E_INVALID = -1
XCT_E_CUDA = -2
XCT_E_NOMEM = -3
XCT_E_UNSUPPORTED = -4
XCT_E_TIMEOUT = -5
XCT_E_IO = -6

FETCH_EXACT = 0
FETCH_AVG2X2 = 1
SUBSETS_REF = 0
SUBSETS_COVER = 1
KERNELS_TILED = 0
KERNELS_PLAIN = 1
PI_OWN_LAYER = 1
FISTA_UPDATE_X = 1
FISTA_ADJOINT = 2
MULTISLICE_SLICES = 8  # slices per group of the slice-interleaved forward projector

# Every function include/xct.h declares (checked by the tests against the header).
EXPORTS = (
    "xct_ctx_create", "xct_ctx_destroy", "xct_device_count", "xct_device_name",
    "xct_osem_plan_create", "xct_osem_plan_destroy", "xct_subset_order",
    "xct_osem_run", "xct_osem_run_device", "xct_fwd", "xct_bp_ref", "xct_adj",
    "xct_plan_sync", "xct_plan_last_ms", "xct_launch_count", "xct_last_error", "xct_abi_version",
    "xct_osem_profile", "xct_fp32_peak", "xct_osem1", "xct_osem2", "xct_osem_run_static",
    "xct_batch_plan_create", "xct_batch_run", "xct_batch_plan_destroy", "xct_osem_run_batched",
    "xct_fbp_filter", "xct_fbp_backproject", "xct_fbp_run_device", "xct_hybrid_run_device", "xct_fbp_run",
    "xct_hybrid_run", "xct_rot_center_shift", "xct_focus_index", "xct_rot_center_search",
    "xct_check_report", "xct_reslice_plan_create", "xct_reslice", "xct_reslice_plan_destroy", "xct_reslice_plan_set_wait_limit",
    "xct_denoise_sinogram",
    "xct_cs_osem_run_device", "xct_cs_osem_run", "xct_plan_autotune", "xct_plan_tuning", "xct_plan_set_tuning",
    "xct_plan_multislice", "xct_plan_set_multislice", "xct_batch_plan_set_cs", "xct_batch_plan_uniform",
    "xct_batch_plan_groups", "xct_batch_plan_set_grouping",
    "xct_fista_power_iteration", "xct_fista_set_lipschitz", "xct_fista_run_device", "xct_fista_run",
    "xct_batch_plan_autotune", "xct_batch_plan_tuning", "xct_osem_run_volume", "xct_hybrid_cs_run_device",
    "xct_hybrid_cs_run",
)

TUNE_FORCE = 1


class XCTError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("xct error %d: %s" % (code, msg))
        self.code = code


class Geom(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("ox", ctypes.c_int), ("oy", ctypes.c_int),
        ("px", ctypes.c_int), ("pa", ctypes.c_int),
        ("ss", ctypes.c_int), ("it", ctypes.c_int),
        ("angles_deg", ctypes.POINTER(ctypes.c_float)),
        ("center_bin", ctypes.c_float),
        ("measured_fetch_mode", ctypes.c_int),
        ("subset_mode", ctypes.c_int),
        ("correction_mode", ctypes.c_int),
        ("max_batch", ctypes.c_int),
        ("kernels", ctypes.c_int),
    ]


_lib = None


def load():
    """Load libxct.so (raises if it was not built: no CPU fallback exists).  With
    XCT_LIB_VARIANT=checked the bounds-checked build libxct_checked.so is loaded instead
    (xct.build.build_lib(checked=True) makes it; check_report reads what it found)."""
    global _lib
    if _lib is not None:
        return _lib
    path = LIB_PATH
    if os.environ.get("XCT_LIB_VARIANT", "") == "checked":
        path = os.path.join(_HERE, "libxct_checked.so")
    if not os.path.exists(path):
        raise XCTError(XCT_E_UNSUPPORTED, "%s not built (run __graft_entry__.build())" % os.path.basename(path))
    L = ctypes.CDLL(path)
    vp, ip, fp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)
    L.xct_ctx_create.argtypes = [ip, ctypes.POINTER(vp)]
    L.xct_ctx_destroy.argtypes = [vp]
    L.xct_device_count.argtypes = [ctypes.POINTER(ctypes.c_int)]
    L.xct_device_name.argtypes = [ip, ctypes.c_char_p, ip]
    L.xct_osem_plan_create.argtypes = [vp, ctypes.POINTER(Geom), ctypes.POINTER(vp)]
    L.xct_osem_plan_destroy.argtypes = [vp]
    L.xct_subset_order.argtypes = [ip, ctypes.POINTER(ctypes.c_int)]
    L.xct_osem_run.argtypes = [vp, ip, ctypes.POINTER(fp), ctypes.POINTER(fp), ctypes.POINTER(ctypes.c_int), ip]
    L.xct_osem_run_device.argtypes = [vp, ip, vp, vp, ctypes.POINTER(ctypes.c_int), ip, vp]
    for n in ("xct_fwd", "xct_bp_ref", "xct_adj"):
        getattr(L, n).argtypes = [vp, ip, vp, vp, vp]
    L.xct_osem_profile.argtypes = [vp, ip, vp, vp, ctypes.POINTER(ctypes.c_int), ip, vp, fp,
                                   ctypes.POINTER(ctypes.c_longlong)]
    L.xct_fp32_peak.argtypes = [ip, fp]
    L.xct_osem1.argtypes = [vp, ip, ip, vp, vp, vp, vp]
    L.xct_osem2.argtypes = [vp, ip, ip, vp, vp, vp]
    L.xct_osem_run_static.argtypes = [ctypes.POINTER(Geom), ip, vp, vp, ctypes.POINTER(ctypes.c_int), ip, vp]
    L.xct_batch_plan_create.argtypes = [vp, ip, ctypes.POINTER(Geom), ip, ctypes.POINTER(vp)]
    L.xct_batch_run.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), vp]
    L.xct_batch_plan_destroy.argtypes = [vp]
    L.xct_osem_run_batched.argtypes = [vp, ip, ctypes.POINTER(Geom), ctypes.POINTER(vp), ctypes.POINTER(vp), ip, vp]
    L.xct_fbp_filter.argtypes = [vp, ip, ip, vp, vp, vp]
    L.xct_fbp_backproject.argtypes = [vp, ip, vp, vp, vp]
    L.xct_fbp_run_device.argtypes = [vp, ip, ip, vp, vp, vp]
    L.xct_hybrid_run_device.argtypes = [vp, ip, ip, ip, vp, vp, ctypes.POINTER(ctypes.c_int), ip, vp]
    L.xct_fbp_run.argtypes = [vp, ip, ip, ctypes.POINTER(fp), ctypes.POINTER(fp)]
    L.xct_hybrid_run.argtypes = [vp, ip, ip, ip, ctypes.POINTER(fp), ctypes.POINTER(fp),
                                 ctypes.POINTER(ctypes.c_int), ip]
    c_f = ctypes.c_float
    L.xct_rot_center_shift.argtypes = [vp, ip, c_f, c_f, vp, vp, vp]
    L.xct_focus_index.argtypes = [vp, ip, ip, c_f, c_f, c_f, c_f, vp, vp, vp]
    L.xct_rot_center_search.argtypes = [vp, ip, c_f, c_f, c_f, c_f, c_f, vp, vp, fp, ctypes.POINTER(ctypes.c_int),
                                        vp]
    L.xct_reslice_plan_create.argtypes = [vp, ip, ip, ip, fp, fp, c_f, ip, ctypes.POINTER(vp)]
    L.xct_reslice.argtypes = [vp, ip, ip, vp, vp, vp]
    L.xct_reslice_plan_destroy.argtypes = [vp]
    L.xct_reslice_plan_set_wait_limit.argtypes = [vp, ctypes.c_longlong]
    L.xct_denoise_sinogram.argtypes = [ip, ip, ip, c_f, vp, vp, vp]
    L.xct_cs_osem_run_device.argtypes = [vp, ip, vp, vp, ctypes.POINTER(ctypes.c_int), ip, c_f, vp]
    L.xct_batch_plan_set_cs.argtypes = [vp, c_f, ip, ctypes.POINTER(ctypes.c_int)]
    L.xct_batch_plan_uniform.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.xct_batch_plan_groups.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.xct_batch_plan_set_grouping.argtypes = [vp, ip]
    L.xct_fista_power_iteration.argtypes = [vp, ip, ip, ip, fp, vp]
    L.xct_fista_set_lipschitz.argtypes = [vp, fp]
    L.xct_fista_run_device.argtypes = [vp, ip, vp, vp, ctypes.POINTER(ctypes.c_int), ip, c_f, c_f, ip, vp]
    L.xct_fista_run.argtypes = [vp, ip, ctypes.POINTER(fp), ctypes.POINTER(fp), ctypes.POINTER(ctypes.c_int), ip, c_f,
                                c_f, ip]
    L.xct_cs_osem_run.argtypes = [vp, ip, ctypes.POINTER(fp), ctypes.POINTER(fp), ctypes.POINTER(ctypes.c_int), ip,
                                  c_f]
    L.xct_hybrid_cs_run_device.argtypes = [vp, ip, ip, ip, vp, vp, ctypes.POINTER(ctypes.c_int), ip, c_f, vp]
    L.xct_hybrid_cs_run.argtypes = [vp, ip, ip, ip, ctypes.POINTER(fp), ctypes.POINTER(fp), ctypes.POINTER(ctypes.c_int),
                                    ip, c_f]
    L.xct_osem_run_volume.argtypes = [vp, ip, ctypes.POINTER(fp), ctypes.POINTER(fp), ctypes.POINTER(ctypes.c_int),
                                      ip]
    L.xct_plan_autotune.argtypes = [vp, ip, ctypes.c_char_p, ip, vp]
    L.xct_plan_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.xct_plan_set_tuning.argtypes = [vp, ip, ip]
    L.xct_plan_multislice.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.xct_plan_set_multislice.argtypes = [vp, ip]
    L.xct_batch_plan_autotune.argtypes = [vp, ctypes.c_char_p, ip, vp]
    L.xct_batch_plan_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.xct_plan_sync.argtypes = [vp]
    L.xct_plan_last_ms.argtypes = [vp, fp]
    L.xct_check_report.argtypes = [vp] + [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int)] + \
        [ctypes.POINTER(ctypes.c_longlong)] * 3
    L.xct_launch_count.restype = ctypes.c_longlong
    L.xct_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def _check(rc):
    if rc != XCT_OK:
        raise XCTError(rc, load().xct_last_error().decode(errors="replace"))


def subset_order(ss):
    """Subset order of OSEM_ocl (GPU.cpp:564-582)."""
    out = (ctypes.c_int * ss)()
    _check(load().xct_subset_order(ss, out))
    return np.array(out[:], dtype=np.int32)


def check_report(ctx):
    """Bounds-checked build only: (skipped accesses since the last report, and the first one's
    site code, index, lower and upper bound); resets the counts."""
    n, site = ctypes.c_longlong(), ctypes.c_int()
    v, lo, hi = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
    _check(load().xct_check_report(ctx.handle, ctypes.byref(n), ctypes.byref(site), ctypes.byref(v),
                                   ctypes.byref(lo), ctypes.byref(hi)))
    return n.value, site.value, v.value, lo.value, hi.value


def launch_count():
    return int(load().xct_launch_count())


def fp32_peak_tflops(device=0):
    """Measured FP32 FMA throughput of the device (TFLOP/s)."""
    v = ctypes.c_float()
    _check(load().xct_fp32_peak(device, ctypes.byref(v)))
    return v.value


def device_count():
    n = ctypes.c_int(0)
    _check(load().xct_device_count(ctypes.byref(n)))
    return n.value


def _ptr(t):
    """Device pointer of a contiguous float32 CUDA tensor (or an int address)."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_contiguous():
        raise XCTError(XCT_E_INVALID, "tensor must be contiguous")
    if str(t.dtype) != "torch.float32":
        raise XCTError(XCT_E_INVALID, "tensor must be float32")
    if not t.is_cuda:
        raise XCTError(XCT_E_INVALID, "tensor must be on a CUDA device")
    return t.data_ptr()


def _need(t, count, what):
    """A buffer handed to the library as a bare pointer must hold the elements the call
    touches: the library cannot see sizes, and a short buffer would be read or written past
    its end on the device."""
    if t is None or isinstance(t, int):
        return
    have = t.numel() if hasattr(t, "numel") else int(np.asarray(t).size)
    if have < count:
        raise XCTError(XCT_E_INVALID, "%s holds %d elements; the call needs %d" % (what, have, count))


def _stream(stream):
    if stream is None:
        try:
            import torch
            return torch.cuda.current_stream().cuda_stream
        except Exception:
            return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Context:
    """One CUDA device (replaces OCL_platform_device for a single device)."""

    def __init__(self, device=0):
        self._lib = load()
        h = ctypes.c_void_p()
        _check(self._lib.xct_ctx_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self._lib.xct_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OSEMPlan:
    """An OS-EM plan: geometry, angle table and device work buffers for up to
    ``max_batch`` slices per call."""

    def __init__(self, ctx, nx, ny, px, angles_deg, ss, it, center_bin=None, fetch_mode=FETCH_EXACT,
                 subset_mode=SUBSETS_REF, correction_mode=0, max_batch=1, kernels=KERNELS_TILED):
        self._lib = load()
        self.ctx = ctx
        self.angles = np.ascontiguousarray(angles_deg, dtype=np.float32)
        self.nx, self.ny, self.px, self.pa, self.ss, self.it = nx, ny, px, int(self.angles.size), ss, it
        self.max_batch = max_batch
        g = Geom(nx, ny, nx, ny, px, self.pa, ss, it,
                 self.angles.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                 -1.0 if center_bin is None else float(center_bin),
                 fetch_mode, subset_mode, correction_mode, max_batch, kernels)
        h = ctypes.c_void_p()
        _check(self._lib.xct_osem_plan_create(ctx.handle, ctypes.byref(g), ctypes.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self._lib.xct_osem_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _sub(self, sub):
        if sub is None:
            return None
        a = (ctypes.c_int * self.ss)(*[int(v) for v in sub])
        return a

    # ---- host arrays (blocking) --------------------------------------------------------
    def run(self, sinos, imgs, sub=None, it=-1):
        """OS-EM on host arrays: ``sinos`` dN float32 [pa][px], ``imgs`` dN float32
        [ny][nx] (initial images in, reconstructions written back in place)."""
        s_arr, i_arr = self._host_arrays(sinos, imgs)
        _check(self._lib.xct_osem_run(self.handle, len(sinos), s_arr, i_arr, self._sub(sub), it))
        return imgs

    def _host_arrays(self, sinos, imgs):
        fp = ctypes.POINTER(ctypes.c_float)
        for a in list(sinos) + list(imgs):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                raise XCTError(XCT_E_INVALID, "host arrays must be C-contiguous float32 numpy arrays")
        if len(imgs) != len(sinos):
            raise XCTError(XCT_E_INVALID, "as many images as sinograms are needed")
        for a in sinos:
            _need(a, self.pa * self.px, "host sinogram")
        for a in imgs:
            _need(a, self.ny * self.nx, "host image")
        dN = len(sinos)
        return (fp * dN)(*[s.ctypes.data_as(fp) for s in sinos]), (fp * dN)(*[i.ctypes.data_as(fp) for i in imgs])

    def run_volume(self, sinos, imgs, sub=None, it=-1):
        """OS-EM of a whole volume from host memory in streamed batches of max_batch slices.
        sinos/imgs: sequences of host slices -- float32 numpy arrays, or CPU torch tensors
        (page-locked ones give overlapped copies)."""
        fp = ctypes.POINTER(ctypes.c_float)

        def addr(a):
            if hasattr(a, "data_ptr"):
                if a.is_cuda or not a.is_contiguous() or str(a.dtype) != "torch.float32":
                    raise XCTError(XCT_E_INVALID, "host slices must be contiguous float32 CPU tensors")
                return ctypes.cast(a.data_ptr(), fp)
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                raise XCTError(XCT_E_INVALID, "host arrays must be C-contiguous float32 numpy arrays")
            return a.ctypes.data_as(fp)
        if len(imgs) != len(sinos):
            raise XCTError(XCT_E_INVALID, "as many images as sinograms are needed")
        for a in sinos:
            _need(a, self.pa * self.px, "host sinogram")
        for a in imgs:
            _need(a, self.ny * self.nx, "host image")
        n = len(sinos)
        s_arr = (fp * n)(*[addr(a) for a in sinos])
        i_arr = (fp * n)(*[addr(a) for a in imgs])
        _check(self._lib.xct_osem_run_volume(self.handle, n, s_arr, i_arr, self._sub(sub), it))
        return imgs

    def cs_run(self, sinos, imgs, cs_lambda=1.0e-4, sub=None, it=-1):
        """Compressed-sensing OS-EM (FISTA_OSEM_execution) on host arrays; the dN slices of
        the call are the third axis of the proximal step."""
        s_arr, i_arr = self._host_arrays(sinos, imgs)
        _check(self._lib.xct_cs_osem_run(self.handle, len(sinos), s_arr, i_arr, self._sub(sub), it, cs_lambda))
        return imgs

    def power_iteration(self, trials=30, work_group=1024, own_layer=False, stream=None):
        """The Lipschitz estimates L[ss] of the subset operators (powerIteration); kept in the
        plan for the FISTA runs.  own_layer: each subset projects its own estimate (the
        reference projects layer 0's for every subset)."""
        out = np.zeros(self.ss, np.float32)
        _check(self._lib.xct_fista_power_iteration(self.handle, trials, work_group,
                                                   PI_OWN_LAYER if own_layer else 0,
                                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                   _stream(stream)))
        return out

    def set_lipschitz(self, L):
        a = np.ascontiguousarray(L, dtype=np.float32)
        if a.size != self.ss:
            raise XCTError(XCT_E_INVALID, "L needs one value per subset")
        _check(self._lib.xct_fista_set_lipschitz(self.handle, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def fista_run(self, sinos, imgs, alpha=1.0, cs_lambda=1.0e-4, sub=None, it=-1, flags=0):
        """FISTA with compressed sensing (FISTA_thread / FISTA_execution) on host arrays;
        reconstructions written into ``imgs`` (their contents are not read)."""
        s_arr, i_arr = self._host_arrays(sinos, imgs)
        _check(self._lib.xct_fista_run(self.handle, len(sinos), s_arr, i_arr, self._sub(sub), it, alpha, cs_lambda,
                                       flags))
        return imgs

    def fbp_run(self, sinos, imgs, zp=0):
        """FBP (FBP_thread) on host arrays; reconstructions written into ``imgs``."""
        s_arr, i_arr = self._host_arrays(sinos, imgs)
        _check(self._lib.xct_fbp_run(self.handle, len(sinos), zp, s_arr, i_arr))
        return imgs

    def hybrid_cs_run(self, sinos, imgs, zp=0, baseup_order=4, cs_lambda=1.0e-4, sub=None, it=-1):
        """FBP + base-up + compressed-sensing OS-EM (hybrid_thread with CSitBool) on host arrays."""
        s_arr, i_arr = self._host_arrays(sinos, imgs)
        _check(self._lib.xct_hybrid_cs_run(self.handle, len(sinos), zp, baseup_order, s_arr, i_arr, self._sub(sub),
                                           it, cs_lambda))
        return imgs

    def hybrid_run(self, sinos, imgs, zp=0, baseup_order=4, sub=None, it=-1):
        """FBP + base-up + OS-EM (hybrid_thread) on host arrays."""
        s_arr, i_arr = self._host_arrays(sinos, imgs)
        _check(self._lib.xct_hybrid_run(self.handle, len(sinos), zp, baseup_order, s_arr, i_arr, self._sub(sub),
                                        it))
        return imgs

    def last_ms(self):
        v = ctypes.c_float()
        _check(self._lib.xct_plan_last_ms(self.handle, ctypes.byref(v)))
        return v.value

    # ---- device tensors (asynchronous on the stream) ----------------------------------
    def run_device(self, d_sino, d_img, dN=None, sub=None, it=-1, stream=None):
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_osem_run_device(self.handle, dN, _ptr(d_sino), _ptr(d_img), self._sub(sub), it,
                                             _stream(stream)))

    def cs_run_device(self, d_sino, d_img, cs_lambda=1.0e-4, dN=None, sub=None, it=-1, stream=None):
        """Compressed-sensing OS-EM on device tensors [dN][pa][px] -> [dN][ny][nx] (in/out)."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_cs_osem_run_device(self.handle, dN, _ptr(d_sino), _ptr(d_img), self._sub(sub), it,
                                                cs_lambda, _stream(stream)))

    def fista_run_device(self, d_sino, d_img, alpha=1.0, cs_lambda=1.0e-4, dN=None, sub=None, it=-1, flags=0,
                         stream=None):
        """FISTA with compressed sensing (FISTA_execution) on device tensors [dN][pa][px] ->
        [dN][ny][nx] (out)."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_fista_run_device(self.handle, dN, _ptr(d_sino), _ptr(d_img), self._sub(sub), it, alpha,
                                              cs_lambda, flags, _stream(stream)))

    def osem1(self, sub, d_img, d_sino, d_ratio, dN=None, stream=None):
        """OSEM1 (OSEM.cl:38-68) alone: ratio rows of subset ``sub`` into d_ratio."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_ratio, dN * self.pa * self.px, "d_ratio")
        _check(self._lib.xct_osem1(self.handle, dN, sub, _ptr(d_img), _ptr(d_sino), _ptr(d_ratio),
                                   _stream(stream)))

    def osem2(self, sub, d_img, d_ratio, dN=None, stream=None):
        """OSEM2 (OSEM.cl:71-105) alone: backprojection of d_ratio + update of d_img."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _need(d_ratio, dN * self.pa * self.px, "d_ratio")
        _check(self._lib.xct_osem2(self.handle, dN, sub, _ptr(d_img), _ptr(d_ratio), _stream(stream)))

    def fwd(self, d_img, d_sino, dN=None, stream=None):
        dN = d_img.shape[0] if dN is None else dN
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _check(self._lib.xct_fwd(self.handle, dN, _ptr(d_img), _ptr(d_sino), _stream(stream)))

    def bp_ref(self, d_sino, d_img, dN=None, stream=None):
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_bp_ref(self.handle, dN, _ptr(d_sino), _ptr(d_img), _stream(stream)))

    def adj(self, d_sino, d_img, dN=None, stream=None):
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_adj(self.handle, dN, _ptr(d_sino), _ptr(d_img), _stream(stream)))

    def fbp_filter(self, d_sino, d_fprj, zp=0, dN=None, stream=None):
        """Ramp-filtered sinograms (FBP.cl:34-160) into d_fprj."""
        dN = d_sino.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_fprj, dN * self.pa * self.px, "d_fprj")
        _check(self._lib.xct_fbp_filter(self.handle, dN, zp, _ptr(d_sino), _ptr(d_fprj), _stream(stream)))

    def fbp_backproject(self, d_fprj, d_img, dN=None, stream=None):
        """backProjectionFBP (FBP.cl:164-188) of filtered sinograms into d_img."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_fprj, dN * self.pa * self.px, "d_fprj")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_fbp_backproject(self.handle, dN, _ptr(d_fprj), _ptr(d_img), _stream(stream)))

    def fbp(self, d_sino, d_img, zp=0, dN=None, stream=None):
        """FBP_execution: (correction), filter, backprojection."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_fbp_run_device(self.handle, dN, zp, _ptr(d_sino), _ptr(d_img), _stream(stream)))

    def hybrid_cs(self, d_sino, d_img, zp=0, baseup_order=4, cs_lambda=1.0e-4, dN=None, sub=None, it=-1,
                  stream=None):
        """FBP + base-up + compressed-sensing OS-EM on device tensors."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_hybrid_cs_run_device(self.handle, dN, zp, baseup_order, _ptr(d_sino), _ptr(d_img),
                                                  self._sub(sub), it, cs_lambda, _stream(stream)))

    def hybrid(self, d_sino, d_img, zp=0, baseup_order=4, dN=None, sub=None, it=-1, stream=None):
        """FBP + base-up + OS-EM of hybrid_thread on device tensors."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        _check(self._lib.xct_hybrid_run_device(self.handle, dN, zp, baseup_order, _ptr(d_sino), _ptr(d_img),
                                               self._sub(sub), it, _stream(stream)))

    # ---- rotation-centre search ---------------------------------------------------------
    def rot_center_shift(self, d_sino, d_shifted, start, step, n=None, stream=None):
        """rotCenterShift of one sinogram [pa][px] for shifts start + step*i -> [n][pa][px]."""
        n = d_shifted.shape[0] if n is None else n
        _need(d_sino, self.pa * self.px, "d_sino")
        _need(d_shifted, n * self.pa * self.px, "d_shifted")
        _check(self._lib.xct_rot_center_shift(self.handle, n, start, step, _ptr(d_sino), _ptr(d_shifted),
                                              _stream(stream)))

    def focus_index(self, d_imgs, d_findex, start, step, ang_ini, ang_fin, offset=0, n=None, stream=None):
        """setMask + imgFocusIndex of images [n][ny][nx] -> d_findex [n] (device)."""
        n = d_imgs.shape[0] if n is None else n
        _need(d_imgs, n * self.ny * self.nx, "d_imgs")
        _need(d_findex, n, "d_findex")
        _check(self._lib.xct_focus_index(self.handle, n, offset, start, step, ang_ini, ang_fin, _ptr(d_imgs),
                                         _ptr(d_findex), _stream(stream)))

    def rot_center_search(self, d_sino, d_imgs, start, step, ang_ini=None, ang_fin=None, init_value=1.0, n=None,
                          stream=None):
        """The whole search; returns (focus indices [n] (numpy), index of the best shift).
        ang_ini/ang_fin default to the plan's first and last angle."""
        n = d_imgs.shape[0] if n is None else n
        _need(d_sino, self.pa * self.px, "d_sino")
        _need(d_imgs, n * self.ny * self.nx, "d_imgs")
        ang_ini = float(self.angles[0]) if ang_ini is None else ang_ini
        ang_fin = float(self.angles[-1]) if ang_fin is None else ang_fin
        fi = np.zeros(n, np.float32)
        best = ctypes.c_int(-1)
        _check(self._lib.xct_rot_center_search(self.handle, n, start, step, ang_ini, ang_fin, init_value,
                                               _ptr(d_sino), _ptr(d_imgs),
                                               fi.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(best),
                                               _stream(stream)))
        return fi, best.value

    # ---- forward-projector tiles --------------------------------------------------------
    def autotune(self, dN=None, cache_path=None, force=False, stream=None):
        """Time every (tile side, angles per CTA) candidate for dN slices and keep the fastest
        (cached per shape in memory and in cache_path / $XCT_TUNE_CACHE)."""
        dN = self.max_batch if dN is None else dN
        cp = None if cache_path is None else str(cache_path).encode()
        _check(self._lib.xct_plan_autotune(self.handle, dN, cp, TUNE_FORCE if force else 0, _stream(stream)))
        return self.tuning()

    def tuning(self):
        t, c = ctypes.c_int(), ctypes.c_int()
        _check(self._lib.xct_plan_tuning(self.handle, ctypes.byref(t), ctypes.byref(c)))
        return t.value, c.value

    def set_tuning(self, fwd_tile, ang_chunk):
        _check(self._lib.xct_plan_set_tuning(self.handle, fwd_tile, ang_chunk))

    def multislice(self):
        """Angle chunk of the slice-interleaved forward projector (0 = off)."""
        v = ctypes.c_int()
        _check(self._lib.xct_plan_multislice(self.handle, ctypes.byref(v)))
        return v.value

    def set_multislice(self, ang_chunk):
        """Turn the slice-interleaved forward projector on (subset angles per CTA, 1..128) or
        off (0) for calls of eight or more slices."""
        _check(self._lib.xct_plan_set_multislice(self.handle, int(ang_chunk)))

    def profile(self, d_sino, d_img, dN=None, sub=None, it=-1, stream=None):
        """Run OS-EM with CUDA events around every launch; returns a dict of summed device
        milliseconds and launch counts per kernel kind (fwd, finalize, bp) and the total."""
        dN = d_img.shape[0] if dN is None else dN
        _need(d_sino, dN * self.pa * self.px, "d_sino")
        _need(d_img, dN * self.ny * self.nx, "d_img")
        ms = (ctypes.c_float * 4)()
        n = (ctypes.c_longlong * 4)()
        _check(self._lib.xct_osem_profile(self.handle, dN, _ptr(d_sino), _ptr(d_img), self._sub(sub), it,
                                          _stream(stream), ms, n))
        keys = ("fwd", "finalize", "bp", "total")
        return {k: {"ms": ms[i], "launches": int(n[i])} for i, k in enumerate(keys)}

    def sync(self):
        _check(self._lib.xct_plan_sync(self.handle))


def make_geom(nx, ny, px, angles_deg, ss, it, center_bin=None, fetch_mode=FETCH_EXACT, subset_mode=SUBSETS_REF,
              correction_mode=0, max_batch=1, kernels=KERNELS_TILED):
    """An xct_geom (keeps the angle array alive on the returned object as ._angles)."""
    ang = np.ascontiguousarray(angles_deg, dtype=np.float32)
    g = Geom(nx, ny, nx, ny, px, int(ang.size), ss, it, ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
             -1.0 if center_bin is None else float(center_bin), fetch_mode, subset_mode, correction_mode,
             max_batch, kernels)
    g._angles = ang
    return g


class BatchPlan:
    """OS-EM over slices of different shapes (same subset count) in one CUDA graph of
    persistent launches (xct_batch_plan_create / xct_batch_run); slices that share one
    geometry, eight or more, run through a single-shape plan of their own (geometry groups)."""

    def __init__(self, ctx, geoms, it):
        self._lib = load()
        self.ctx = ctx
        self.geoms = list(geoms)
        arr = (Geom * len(self.geoms))(*self.geoms)
        h = ctypes.c_void_p()
        _check(self._lib.xct_batch_plan_create(ctx.handle, len(self.geoms), arr, it, ctypes.byref(h)))
        self.handle = h

    def autotune(self, cache_path=None, force=False, stream=None):
        cp = None if cache_path is None else str(cache_path).encode()
        _check(self._lib.xct_batch_plan_autotune(self.handle, cp, TUNE_FORCE if force else 0, _stream(stream)))
        return self.tuning()

    def tuning(self):
        t, c = ctypes.c_int(), ctypes.c_int()
        _check(self._lib.xct_batch_plan_tuning(self.handle, ctypes.byref(t), ctypes.byref(c)))
        return t.value, c.value

    def uniform(self):
        """Slices per call when every slice is in one geometry group (0: not so)."""
        v = ctypes.c_int()
        _check(self._lib.xct_batch_plan_uniform(self.handle, ctypes.byref(v)))
        return v.value

    def groups(self):
        """(number of geometry groups, slices they hold)."""
        g, k = ctypes.c_int(), ctypes.c_int()
        _check(self._lib.xct_batch_plan_groups(self.handle, ctypes.byref(g), ctypes.byref(k)))
        return g.value, k.value

    def set_grouping(self, on):
        """Geometry groups on (the default) or off (the graph serves every slice)."""
        _check(self._lib.xct_batch_plan_set_grouping(self.handle, 1 if on else 0))

    def run(self, sinos, imgs, stream=None):
        n = len(self.geoms)
        if len(sinos) != n or len(imgs) != n:
            raise XCTError(XCT_E_INVALID, "one sinogram and one image per item are needed")
        for g, a, b in zip(self.geoms, sinos, imgs):
            _need(a, g.pa * g.px, "item sinogram")
            _need(b, g.ny * g.nx, "item image")
        s = (ctypes.c_void_p * n)(*[_ptr(t) for t in sinos])
        i = (ctypes.c_void_p * n)(*[_ptr(t) for t in imgs])
        _check(self._lib.xct_batch_run(self.handle, s, i, _stream(stream)))

    def set_cs(self, stack_len, cs_lambda=1.0e-4):
        """Compressed-sensing OS-EM over stacks of consecutive slices of one image size
        (stack_len: the stacks' lengths in slice order; empty turns it off).  Each stack's
        images must then be consecutive in one array when the plan runs."""
        lens = [int(v) for v in stack_len]
        arr = (ctypes.c_int * max(1, len(lens)))(*lens)
        _check(self._lib.xct_batch_plan_set_cs(self.handle, float(cs_lambda), len(lens), arr))

    def close(self):
        if self.handle:
            self._lib.xct_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ReslicePlan:
    """Projection stack -> sinograms on the device (Reslice/reslice_ocl.cpp reslice())."""

    def __init__(self, ctx, width, height, n_angles, xshift=None, yshift=None, baseup=0.0, correction=0):
        self._lib = load()
        self.ctx = ctx
        self.width, self.height, self.n_angles = width, height, n_angles
        fp = ctypes.POINTER(ctypes.c_float)
        xs = None if xshift is None else np.ascontiguousarray(xshift, dtype=np.float32)
        ys = None if yshift is None else np.ascontiguousarray(yshift, dtype=np.float32)
        for a in (xs, ys):
            if a is not None and a.size != n_angles:
                raise XCTError(XCT_E_INVALID, "shift arrays must have n_angles entries")
        h = ctypes.c_void_p()
        _check(self._lib.xct_reslice_plan_create(ctx.handle, width, height, n_angles,
                                                 None if xs is None else xs.ctypes.data_as(fp),
                                                 None if ys is None else ys.ctypes.data_as(fp),
                                                 baseup, correction, ctypes.byref(h)))
        self.handle = h

    def reslice(self, d_proj, d_sino, first_angle=0, n=None, stream=None):
        """d_proj [n][height][width] (angles first_angle..) -> rows of d_sino [height][n_angles][width]."""
        n = d_proj.shape[0] if n is None else n
        _need(d_proj, n * self.height * self.width, "d_proj")
        _need(d_sino, self.height * self.n_angles * self.width, "d_sino")
        _check(self._lib.xct_reslice(self.handle, first_angle, n, _ptr(d_proj), _ptr(d_sino), _stream(stream)))

    def set_wait_limit(self, sm_clocks):
        """Diagnostics: limit of the staged kernel's waits for its tile copies (SM clocks); a
        negative value makes every wait give up at once (global-memory fallback)."""
        _check(self._lib.xct_reslice_plan_set_wait_limit(self.handle, int(sm_clocks)))

    def close(self):
        """Destroys the plan; raises XCTError (XCT_E_TIMEOUT) if a staged-window copy of any
        reslice call missed its wait limit (those tiles were computed from global memory)."""
        if self.handle:
            h, self.handle = self.handle, None
            _check(self._lib.xct_reslice_plan_destroy(h))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def denoise_sinogram(d_src, d_dst, threshold, stream=None):
    """denoiseSinogram (Reslice/reslice.cl:223-248) on sinograms [rows][angles][width]."""
    rows, na, w = d_src.shape
    _need(d_dst, rows * na * w, "d_dst")
    _check(load().xct_denoise_sinogram(w, na, rows, threshold, _ptr(d_src), _ptr(d_dst), _stream(stream)))


# ---------------------------------------------------------------- reference-named mirrors
def OSEM_execution(plan, sub, reconst_img, prj_img, dN, it, prjCorrection=True, stream=None):
    """Mirror of ``int OSEM_execution(queue, kernels, angle_buffer, int *sub,
    Image2DArray reconst_img, Image2DArray prj_img, int dN, int it, bool prjCorrection)``
    (CT_reconstruction.hpp:77, GPU.cpp:125-240) on device tensors: reconst_img [dN][ny][nx]
    is updated in place from prj_img [dN][pa][px].  The sinogram correction is part of the
    plan (correction_mode); prjCorrection=False runs with it disabled only if the plan's
    mode is 0.  Returns 0."""
    if not prjCorrection and plan is not None and getattr(plan, "_correction", 0):
        raise XCTError(XCT_E_INVALID, "plan was built with a sinogram correction mode")
    plan.run_device(prj_img, reconst_img, dN=dN, sub=sub, it=it, stream=stream)
    return 0


def FISTA_OSEM_execution(plan, sub, reconst_img, prj_img, dN, it, prjCorrection=True, cs_lambda=1.0e-4,
                         stream=None):
    """Mirror of ``int FISTA_OSEM_execution(queue, kernels, angle_buffer, int *sub,
    Image2DArray reconst_img, Image2DArray prj_img, int dN, int it, bool prjCorrection)``
    (CT_reconstruction.hpp, GPU.cpp:243-405) on device tensors; CSlambda is cs_lambda.
    Returns 0."""
    if not prjCorrection and plan is not None and getattr(plan, "_correction", 0):
        raise XCTError(XCT_E_INVALID, "plan was built with a sinogram correction mode")
    plan.cs_run_device(prj_img, reconst_img, cs_lambda=cs_lambda, dN=dN, sub=sub, it=it, stream=stream)
    return 0


def FBP_execution(plan, reconst_img, prj_img, dN, prjCorrection=True, zp=0, stream=None):
    """Mirror of ``int FBP_execution(queue, kernels, angle_buffer, Image2DArray reconst_img,
    Image2DArray prj_img, int dN, bool prjCorrection, unsigned int iter)``
    (CT_reconstruction.hpp, GPU.cpp:665-819) on device tensors; the transform length is zp
    (the reference passes log2 of it as ``iter``).  The sinogram correction is the plan's.
    Returns 0."""
    if not prjCorrection and plan is not None and getattr(plan, "_correction", 0):
        raise XCTError(XCT_E_INVALID, "plan was built with a sinogram correction mode")
    plan.fbp(prj_img, reconst_img, zp=zp, dN=dN, stream=stream)
    return 0


def OSEM_thread(plan, sub, imgs, prjs, startN, endN, it):
    """Mirror of OSEM_thread (CT_reconstruction.hpp:88-90, GPU.cpp:408-476) without the
    output thread: imgs[i] and prjs[i] for slices startN..endN are host arrays; the
    reconstructions are written back into imgs.  Returns 0."""
    dN = endN - startN + 1
    plan.run(list(prjs[:dN]), list(imgs[:dN]), sub=sub, it=it)
    return 0
