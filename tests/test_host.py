"""The C++ drop-in program xct_ct_reconstruction: the reference's .inp keys, file formats and
slice naming (CPU), and an end-to-end reconstruction from files (GPU)."""
import json
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def host_bin(xct_lib):
    from xct import build
    return build.build_host()


# an .inp as the reference reads it: key lines, values on the next line (CRLF on some)
INP_KEYS = [
    ("#Open CL Platform & Device No", "1"),
    ("#Number of Parallel processing per one device", "{par}"),
    ("#測定ファイルディレクトリパス", "{d1}"),
    ("#測定ファイル名", "s****.raw"),
    ("#出力ファイルディレクトリパス", "{d2}"),
    ("#出力ファイル名", "rec_****.img"),
    ("#ログファイルパス", "{f3}"),
    ("#レイヤー数", "{layers}"),
    ("#開始ナンバー", "7"),
    ("#初期画像の使用 1:Yes 2: No", "2"),
    ("#カメラピクセル数", "{px}"),
    ("#投影数", "{pa}"),
    ("#再構成画像サイズ", "{n}"),
    ("#再構成法", "{method}"),
    ("#反復回数", "{it}"),
    ("#サブセット(OSEM)", "{ss}"),
    ("#投影像補正 0:なし 1: x方向のみ 2:θ方向のみ 3:x,θ方向両方", "0"),
]


def write_inp(path, extra=(), **kw):
    kw.setdefault("method", 6)
    kw.setdefault("layers", 3)
    kw.setdefault("par", 4)
    with open(path, "wb") as f:
        for i, (k, v) in enumerate(list(INP_KEYS) + list(extra)):
            eol = b"\r\n" if i % 3 == 0 else b"\n"
            f.write(k.encode("utf-8") + eol + v.format(**kw).encode("utf-8") + eol)


def test_inp_keys_parse_like_the_reference(host_bin, tmp_path):
    p = tmp_path / "a.inp"
    write_inp(p, d1="in dir", d2="out", f3="angles.log", px=96, pa=60, n=80, it=3, ss=5)
    out = subprocess.run([host_bin, "--print-params", str(p)], capture_output=True, text=True, check=True)
    prm = json.loads(out.stdout.strip().splitlines()[-1])
    assert prm["devList"] == "1" and prm["numParallel"] == 4
    assert prm["d1"] == "in dir" and prm["d2"] == "out" and prm["f3"] == "angles.log"
    assert (prm["num"], prm["st"], prm["fst"]) == (3, 7, 2)
    assert (prm["px"], prm["pa"], prm["nx"], prm["ny"], prm["ox"], prm["oy"]) == (96, 60, 80, 80, 80, 80)
    assert (prm["mode"], prm["it"], prm["ss"], prm["correctionMode"]) == (6, 3, 5, 0)
    # untouched keys keep the reference's defaults (main.cpp:12-47)
    assert prm["zp"] == 4096 and prm["CSitBool"] is False and prm["f4"] == "1st.img"
    # <base>####<tail> naming (GPU.cpp:27-34, :497)
    assert prm["first_input"] == "s0007.raw" and prm["first_output"] == "rec_0007.img"


@pytest.mark.parametrize("lst,n,want", [("1", 1, "0"), ("1,2-4", 8, "0,1,2,3"), ("2", 1, ""),
                                        ("1-3,5", 6, "0,1,2,4"), ("3,1", 4, "0,2")])
def test_device_list_syntax(host_bin, lst, n, want):
    out = subprocess.run([host_bin, "--devlist", lst, str(n)], capture_output=True, text=True, check=True)
    assert out.stdout.strip() == want


def test_input_failures_stop_before_any_reconstruction(host_bin, tmp_path):
    """Missing input directory or first sinogram (main.cpp:76-108: exit 255), a missing angle
    file, and an angle file shorter than the projection count stop the program with a
    message before any device work."""
    d1, d2 = tmp_path / "in", tmp_path / "out"
    inp = tmp_path / "run.inp"
    kw = dict(d1=str(d1), d2=str(d2), f3=str(tmp_path / "angles.log"), px=16, pa=10, n=16, it=1, ss=2)
    write_inp(inp, **kw)
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 255 and "Directory not found" in r.stdout
    d1.mkdir()
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 255 and "No raw file found" in r.stdout
    for z in range(7, 10):
        np.zeros(16 * 10, np.float32).tofile(d1 / ("s%04d.raw" % z))
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "angles.log" in r.stderr
    with open(tmp_path / "angles.log", "w") as f:
        for k in range(9):  # one short
            f.write("%g\n" % (k * 18.0))
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "line 10 holds no angle" in r.stderr
    assert not d2.exists()


@pytest.mark.gpu
def test_end_to_end_reconstruction_from_files(host_bin, oracle_lib, tmp_path):
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, ss, it = 80, 96, 60, 5, 3
    ang = P.uniform_angles(pa)
    d1, d2 = tmp_path / "in", tmp_path / "out"
    d1.mkdir()
    with open(tmp_path / "angles.log", "w") as f:
        for a in ang:
            f.write("%.9g\t0.0\n" % a)  # first token per line (fileIO.cpp:11-23)
    meas = {}
    for z in range(7, 10):
        img = P.rasterize_ellipses(P.ellipse_params(n, 5, z, axes=(3, 20)), n, n)
        meas[z] = P.noisy_log_sinogram(O.projection(img, ang, px), 1e5, z)
        meas[z].astype(np.float32).tofile(d1 / ("s%04d.raw" % z))
    inp = tmp_path / "run.inp"
    write_inp(inp, d1=str(d1), d2=str(d2), f3=str(tmp_path / "angles.log"), px=px, pa=pa, n=n, it=it, ss=ss)
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    x0 = np.ones((n, n), np.float32)
    for z in range(7, 10):
        got = np.fromfile(d2 / ("rec_%04d.img" % z), np.float32).reshape(n, n)
        ref = O.osem_run(x0, meas[z], ang, ss, it, order=O.ORDER_LITERAL)
        rel = np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert rel <= 1e-4, (z, rel)


@pytest.mark.gpu
def test_initial_image_from_file(host_bin, oracle_lib, tmp_path):
    """g_fst = 1: every slice starts from the raw float32 image named by the initial-image
    key (first_image, fileIO.cpp:55-68), here an absolute path."""
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, ss, it = 64, 72, 45, 5, 2
    ang = P.uniform_angles(pa)
    d1, d2 = tmp_path / "in", tmp_path / "out"
    d1.mkdir()
    with open(tmp_path / "angles.log", "w") as f:
        for a in ang:
            f.write("%.9g\n" % a)
    meas = {}
    for z in range(7, 10):
        img = P.rasterize_ellipses(P.ellipse_params(n, 4, z, axes=(3, 16)), n, n)
        meas[z] = P.noisy_log_sinogram(O.projection(img, ang, px), 1e5, z)
        meas[z].astype(np.float32).tofile(d1 / ("s%04d.raw" % z))
    x0 = np.random.default_rng(2).uniform(0.5, 1.5, (n, n)).astype(np.float32)
    x0.tofile(tmp_path / "start.img")
    keys = [("#初期画像の使用 1:Yes 2: No", "1"), ("#初期画像ファイル名", str(tmp_path / "start.img"))]
    inp = tmp_path / "run.inp"
    write_inp(inp, extra=keys, d1=str(d1), d2=str(d2), f3=str(tmp_path / "angles.log"), px=px, pa=pa, n=n, it=it,
              ss=ss)
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    for z in range(7, 10):
        got = np.fromfile(d2 / ("rec_%04d.img" % z), np.float32).reshape(n, n)
        ref = O.osem_run(x0, meas[z], ang, ss, it, order=O.ORDER_LITERAL)
        rel = np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert rel <= 1e-4, (z, rel)
    # a missing initial image is an error, not a silent uniform start
    os.remove(tmp_path / "start.img")
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode != 0 and "start.img" in (r.stdout + r.stderr)


@pytest.mark.gpu
@pytest.mark.parametrize("method", [7, 8])
def test_fbp_and_hybrid_methods_from_files(host_bin, oracle_lib, tmp_path, method):
    """Methods 7 (FBP) and 8 (FBP + OS-EM hybrid) of GPU() (GPU.cpp:80-90) with the .inp's
    zero padding and base-up order keys."""
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, ss, it, zp, order = 64, 72, 45, 3, 2, 256, 3
    ang = P.uniform_angles(pa)
    d1, d2 = tmp_path / "in", tmp_path / "out"
    d1.mkdir()
    with open(tmp_path / "angles.log", "w") as f:
        for a in ang:
            f.write("%.9g\n" % a)
    meas = {}
    for z in range(7, 10):
        img = P.rasterize_ellipses(P.ellipse_params(n, 5, z, axes=(3, 16)), n, n)
        meas[z] = P.noisy_log_sinogram(O.projection(img, ang, px), 1e5, z)
        meas[z].astype(np.float32).tofile(d1 / ("s%04d.raw" % z))
    inp = tmp_path / "run.inp"
    write_inp(inp, extra=[("#ゼロパディングサイズ(FBP)", str(zp)), ("#Base up 減少速度次数 (Hybrid)", str(order))],
              d1=str(d1), d2=str(d2), f3=str(tmp_path / "angles.log"), px=px, pa=pa, n=n, it=it, ss=ss,
              method=method)
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    for z in range(7, 10):
        got = np.fromfile(d2 / ("rec_%04d.img" % z), np.float32).reshape(n, n)
        ref = O.fbp(meas[z], ang, n, n, zp)
        if method == 8:
            ref = O.osem_run(O.base_up(ref, order)[0], meas[z], ang, ss, it, order=O.ORDER_LITERAL)
        rel = np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert rel <= (2e-5 if method == 7 else 1e-4), (z, rel)


@pytest.mark.gpu
@pytest.mark.parametrize("method", [1, 3])
def test_fista_batches_from_files(host_bin, oracle_lib, tmp_path, method):
    """Methods 1 (AART) and 3 (ASIRT) with CSitBool: FISTA_ocl -- the power iteration once per
    device, then FISTA_execution on overlapping batches of 4 slices (overlap 1), as the
    compressed-sensing OS-EM dispatches them (GPU.cpp:2258-2276).  Method 3 uses one subset."""
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, ss, it = 48, 48, 40, 4, 2
    ang = P.uniform_angles(pa)
    d1, d2 = tmp_path / "in", tmp_path / "out"
    d1.mkdir()
    with open(tmp_path / "angles.log", "w") as f:
        for a in ang:
            f.write("%.9g\n" % a)
    prm = P.ellipsoid_params(n, 6, count=5, seed=19)
    meas = {}
    for z in range(7, 13):
        meas[z] = P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z - 7, n, n), ang, px), 1e4, z)
        meas[z].astype(np.float32).tofile(d1 / ("s%04d.raw" % z))
    inp = tmp_path / "run.inp"
    keys = [("#逐次圧縮センシング計算 (FBP適応外)", "1"), ("#逐次圧縮センシング計算加算ファクター", "0.0002"),
            ("#逐次圧縮センシング計算重複レイヤー数", "1"), ("#AARTファクター", "0.8")]
    write_inp(inp, extra=keys, d1=str(d1), d2=str(d2), f3=str(tmp_path / "angles.log"), px=px, pa=pa, n=n, it=it,
              ss=ss, layers=6, par=4, method=method)
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    s_used = ss if method == 1 else 1
    L = O.power_iteration(ang, n, n, px, s_used, trials=30)

    def batch(zs):
        return O.fista_run(np.zeros((len(zs), n, n)), np.stack([meas[z] for z in zs]), ang, s_used, it, L, 0.8, 2e-4)
    b1, b2, b3 = batch(range(7, 11)), batch(range(9, 13)), batch(range(11, 13))
    want = {7: b1[0], 8: b1[1], 9: b1[2], 10: b2[1], 11: b2[2], 12: b3[1]}
    for z, ref in want.items():
        got = np.fromfile(d2 / ("rec_%04d.img" % z), np.float32).reshape(n, n)
        rel = np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert rel <= 1e-4, (z, rel)


@pytest.mark.gpu
@pytest.mark.parametrize("method", [6, 8])
def test_compressed_sensing_batches_from_files(host_bin, oracle_lib, tmp_path, method):
    """CSitBool with 4 slices per call overlapping by 1 (GPU.cpp:636-647, 449-460; the hybrid's
    dispatcher likewise, :1718-1734): slices 7..12 run as batches [7..10], [9..12] and -- the
    dispatcher steps by dN - 2 while the start is in range -- [11..12]; each slice file holds
    the batch that writes it last.  Method 6: OS-EM; method 8: FBP, base-up, then the
    compressed-sensing OS-EM (hybrid_thread, :1569-1571)."""
    from xct import phantom as P
    O = oracle_lib
    n, px, pa, ss, it = 48, 48, 40, 4, 2
    ang = P.uniform_angles(pa)
    d1, d2 = tmp_path / "in", tmp_path / "out"
    d1.mkdir()
    with open(tmp_path / "angles.log", "w") as f:
        for a in ang:
            f.write("%.9g\n" % a)
    prm = P.ellipsoid_params(n, 6, count=5, seed=9)
    meas = {}
    for z in range(7, 13):
        meas[z] = P.noisy_log_sinogram(O.projection(P.ellipsoid_slice(prm, z - 7, n, n), ang, px), 1e4, z)
        meas[z].astype(np.float32).tofile(d1 / ("s%04d.raw" % z))
    inp = tmp_path / "run.inp"
    keys = [("#逐次圧縮センシング計算 (FBP適応外)", "1"), ("#逐次圧縮センシング計算加算ファクター", "0.0002"),
            ("#逐次圧縮センシング計算重複レイヤー数", "1")]
    keys += [("#ゼロパディングサイズ(FBP)", "128"), ("#Base up 減少速度次数 (Hybrid)", "4")]
    write_inp(inp, extra=keys, d1=str(d1), d2=str(d2), f3=str(tmp_path / "angles.log"), px=px, pa=pa, n=n, it=it,
              ss=ss, layers=6, par=4, method=method)
    r = subprocess.run([host_bin, str(inp)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    def batch(zs):
        if method == 6:
            x0 = np.ones((len(zs), n, n), np.float32)
        else:
            x0 = np.stack([O.base_up(O.fbp(meas[z], ang, n, n, 128), 4)[0] for z in zs])
        return O.cs_osem_run(x0, np.stack([meas[z] for z in zs]), ang, ss, it, 2e-4)
    b1, b2, b3 = batch(range(7, 11)), batch(range(9, 13)), batch(range(11, 13))
    want = {7: b1[0], 8: b1[1], 9: b1[2], 10: b2[1], 11: b2[2], 12: b3[1]}
    for z, ref in want.items():
        got = np.fromfile(d2 / ("rec_%04d.img" % z), np.float32).reshape(n, n)
        rel = np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert rel <= 1e-4, (z, rel)
