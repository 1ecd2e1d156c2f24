"""Recipe for oracle/_ref: the reference's own OpenCL kernels compiled on the host.

TEST INFRASTRUCTURE ONLY.  The reference (NozomuIshiguro/CT-XAFS_analysis) has no tests
and no CPU build; its kernels are OpenCL C JIT-compiled at run time with the problem shape
as -D macros (CT_reconstruction/GPU.cpp:537-550).  This recipe compiles
CT_reconstruction/FBP.cl, OSEM.cl, FISTA.cl, AART.cl and reconstShare.cl (OSEM_programBuild builds
OSEM, FISTA and reconstShare as one program, GPU.cpp:527-535; FISTA_programBuild AART, FISTA and
reconstShare, GPU.cpp:2032-2047), where they lie in the reference checkout, with g++ against oracle/ref_shim/cl_shim.hpp (an
OpenCL-C environment written for this project).  The only changes to the kernel text are
mechanical and happen in the build output: OpenCL vector literals ``(float4)(a,b,c,d)``
become constructor calls ``float4(a,b,c,d)`` (C++ would parse the former as a comma
expression), the two-component swizzles ``v.xx`` / ``v.yy`` / ``v.yx`` become member calls
``v.xx()`` etc., and the bare address-space qualifier ``global`` becomes ``__global``.  The
FBP program is built with -D ZP_SIZE as the reference builds it (GPU.cpp:947-954).  The generated
translation unit and the shared objects go to oracle/_ref/ (git-ignored), one library per
problem shape, exactly as the reference JIT-builds one program per shape.

The reference checkout is only present where the project is developed; on a machine
without it ``available()`` is False and the tests that use this build skip.
"""
import os
import re
import subprocess
import hashlib

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: XCT_REFERENCE_ROOT, else a sibling directory "reference" of the repository
REF_ROOT = os.environ.get("XCT_REFERENCE_ROOT") or os.path.join(os.path.dirname(HERE), "..", "reference")
OUT = os.path.join(HERE, "_ref")
KERNELS = ("CT_reconstruction/FBP.cl", "CT_reconstruction/OSEM.cl", "CT_reconstruction/FISTA.cl",
           "CT_reconstruction/AART.cl", "CT_reconstruction/reconstShare.cl")
_VEC = re.compile(r"\((float|int|uint)([234])\)\s*\(")
_SWZ = re.compile(r"\.(xx|yy|yx)\b")
_GLOBAL = re.compile(r"(?<![_\w])global(?=\s)")


def available():
    return all(os.path.isfile(os.path.join(REF_ROOT, k)) for k in KERNELS)


def _rewrite(text):
    text = text.lstrip("﻿")
    text = _VEC.sub(lambda m: "%s%s(" % (m.group(1), m.group(2)), text)
    text = _SWZ.sub(lambda m: ".%s()" % m.group(1), text)
    return _GLOBAL.sub("__global", text)


def default_zp(px):
    """Smallest power of two >= 2*px (4096 for 2048 bins, the reference's default g_zp)."""
    zp = 1
    while zp < 2 * px:
        zp *= 2
    return zp


def build(nx, ny, px, pa, ss, zp=None, force=False, cs_lambda="0.0001"):
    """Compile the reference kernels for one shape; return the .so path.  cs_lambda is the
    text of -D LAMBDA_FISTA (the reference streams the float CSlambda, GPU.cpp:549)."""
    zp = default_zp(px) if zp is None else int(zp)
    if not available():
        raise FileNotFoundError("reference kernel sources not found under %s" % REF_ROOT)
    os.makedirs(OUT, exist_ok=True)
    parts = ['#include "%s"' % os.path.join(HERE, "ref_shim", "cl_shim.hpp"), "namespace clk {"]
    for k in KERNELS:
        with open(os.path.join(REF_ROOT, k), encoding="utf-8") as f:
            parts.append("// ---- %s (vector literals rewritten) ----" % k)
            parts.append(_rewrite(f.read()))
    parts.append("}  // namespace clk")
    parts.append('#include "%s"' % os.path.join(HERE, "ref_shim", "ref_driver.inc"))
    src = "\n".join(parts) + "\n"
    tag = "%dx%d_%dx%d_s%d_zp%d_l%s" % (nx, ny, px, pa, ss, zp, cs_lambda)
    h = hashlib.sha1(src.encode())
    for dep in ("cl_shim.hpp", "ref_driver.inc"):
        with open(os.path.join(HERE, "ref_shim", dep), "rb") as f:
            h.update(f.read())
    digest = h.hexdigest()[:10]
    cpp = os.path.join(OUT, "ref_kernels_%s.cpp" % tag)
    so = os.path.join(OUT, "libref_%s_%s.so" % (tag, digest))
    if os.path.exists(so) and not force:
        return so
    with open(cpp, "w") as f:
        f.write(src)
    defs = [
        "-DIMAGESIZE_X=%d" % nx, "-DIMAGESIZE_Y=%d" % ny, "-DIMAGESIZE_M=%d" % (nx * ny),
        "-DDEPTHSIZE=%d" % max(nx, ny), "-DPRJ_IMAGESIZE=%d" % px, "-DPRJ_ANGLESIZE=%d" % pa,
        "-DPRJ_IMAGESIZE_M=%d" % (px * pa), "-DSS=%d" % ss, "-DLAMBDA_FISTA=%s" % cs_lambda, "-DZP_SIZE=%d" % zp,
    ]
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC",
           "-w", "-o", so, cpp] + defs
    subprocess.run(cmd, check=True)
    return so


if __name__ == "__main__":
    import sys
    shape = [int(v) for v in sys.argv[1:6]] if len(sys.argv) >= 6 else [64, 64, 64, 90, 10]
    print(build(*shape))


RCS_KERNEL = "RotationCenterSearch/rotCenterSearch.cl"


def rcs_available():
    return os.path.isfile(os.path.join(REF_ROOT, RCS_KERNEL))


def build_rcs(width, height, force=False):
    """Compile RotationCenterSearch/rotCenterSearch.cl for one image size (the -D size
    macros the reference leaves at their 2048 defaults); return the .so path."""
    if not rcs_available():
        raise FileNotFoundError("reference kernel sources not found under %s" % REF_ROOT)
    os.makedirs(OUT, exist_ok=True)
    parts = ['#include "%s"' % os.path.join(HERE, "ref_shim", "cl_shim.hpp"), "namespace clk {"]
    with open(os.path.join(REF_ROOT, RCS_KERNEL), encoding="utf-8") as f:
        parts.append("// ---- %s (vector literals rewritten) ----" % RCS_KERNEL)
        parts.append(_rewrite(f.read()))
    parts.append("}  // namespace clk")
    parts.append('#include "%s"' % os.path.join(HERE, "ref_shim", "rcs_driver.inc"))
    src = "\n".join(parts) + "\n"
    tag = "%dx%d" % (width, height)
    h = hashlib.sha1(src.encode())
    for dep in ("cl_shim.hpp", "rcs_driver.inc"):
        with open(os.path.join(HERE, "ref_shim", dep), "rb") as f:
            h.update(f.read())
    digest = h.hexdigest()[:10]
    cpp = os.path.join(OUT, "rcs_kernels_%s.cpp" % tag)
    so = os.path.join(OUT, "librcs_%s_%s.so" % (tag, digest))
    if os.path.exists(so) and not force:
        return so
    with open(cpp, "w") as f:
        f.write(src)
    defs = ["-DIMAGESIZE_X=%d" % width, "-DIMAGESIZE_Y=%d" % height, "-DIMAGESIZE_M=%d" % (width * height)]
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-ffp-contract=off", "-Wno-narrowing", "-shared", "-fPIC",
           "-w", "-o", so, cpp] + defs
    subprocess.run(cmd, check=True)
    return so


RESLICE_KERNEL = "Reslice/reslice.cl"


def reslice_available():
    return os.path.isfile(os.path.join(REF_ROOT, RESLICE_KERNEL))


def build_reslice(width, height, n_angles, force=False):
    """Compile Reslice/reslice.cl for one (width, height, angles) with the -D options of
    reslice_programBuild (Reslice/reslice_ocl.cpp:429-435); return the .so path."""
    if not reslice_available():
        raise FileNotFoundError("reference kernel sources not found under %s" % REF_ROOT)
    os.makedirs(OUT, exist_ok=True)
    parts = ['#include "%s"' % os.path.join(HERE, "ref_shim", "cl_shim.hpp"), "namespace clk {"]
    with open(os.path.join(REF_ROOT, RESLICE_KERNEL), encoding="utf-8") as f:
        parts.append("// ---- %s (vector literals rewritten) ----" % RESLICE_KERNEL)
        parts.append(_rewrite(f.read()))
    parts.append("}  // namespace clk")
    parts.append('#include "%s"' % os.path.join(HERE, "ref_shim", "reslice_driver.inc"))
    src = "\n".join(parts) + "\n"
    tag = "%dx%d_a%d" % (width, height, n_angles)
    h = hashlib.sha1(src.encode())
    for dep in ("cl_shim.hpp", "reslice_driver.inc"):
        with open(os.path.join(HERE, "ref_shim", dep), "rb") as f:
            h.update(f.read())
    digest = h.hexdigest()[:10]
    cpp = os.path.join(OUT, "reslice_kernels_%s.cpp" % tag)
    so = os.path.join(OUT, "libreslice_%s_%s.so" % (tag, digest))
    if os.path.exists(so) and not force:
        return so
    with open(cpp, "w") as f:
        f.write(src)
    defs = ["-DPRJ_ANGLESIZE=%d" % n_angles, "-DNUM_TRIAL=20", "-DLAMBDA=0.001f", "-DIMAGESIZE_X=%d" % width,
            "-DIMAGESIZE_Y=%d" % height, "-DIMAGESIZE_M=%d" % (width * height)]
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-Wno-narrowing", "-shared", "-fPIC",
           "-w", "-o", so, cpp] + defs
    subprocess.run(cmd, check=True)
    return so
