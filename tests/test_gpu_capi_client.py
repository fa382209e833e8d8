"""A C++ host program bound through include/gd2d.h and the CUDA runtime alone
(tests/capi_client.cpp, built here with g++ against the in-tree libgd2d.so) runs the
reference's main-loop protocol -- gd_step_ref into the other buffer, gd_funk_time, twice per
iteration -- on device buffers it allocates itself; its final state, dt and time equal the
same protocol driven from Python through the ctypes mirror, bit for bit, for both physics
and both modes."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ITERS = 5


def build_client(tmp_path):
    cxx = shutil.which("g++")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    inc, lib = os.path.join(cuda, "include"), os.path.join(cuda, "lib64")
    if cxx is None or not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA runtime headers are missing")
    pkg = os.path.dirname(g.lib_path())
    exe = str(tmp_path / "capi_client")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", inc,
                    os.path.join(ROOT, "tests", "capi_client.cpp"), "-o", exe, "-L", pkg,
                    "-lgd2d", "-L", lib, "-lcudart", f"-Wl,-rpath,{pkg}", f"-Wl,-rpath,{lib}"],
                   check=True, capture_output=True, text=True)
    return exe


def python_loop(cfg, s, u, b):
    import torch
    sol = g.Solver(cfg)
    dev = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()
    s, u, b = dev(s), dev(u), dev(b)
    s2, u2 = torch.zeros_like(s), torch.zeros_like(u)
    b2 = None if b is None else torch.zeros_like(b)
    T = torch.tensor([1e7], dtype=torch.float64, device="cuda")
    T_do = torch.tensor([1e-4], dtype=torch.float64, device="cuda")
    TT = torch.tensor([0.0], dtype=torch.float64, device="cuda")
    i = torch.tensor([0], dtype=torch.int32, device="cuda")
    for it in range(ITERS):
        sol.kernel_step(s, u, b, s2, u2, b2, T, T_do, it)
        sol.funk_time(T, T_do, TT, i)
        sol.kernel_step(s2, u2, b2, s, u, b, T, T_do, it)
        sol.funk_time(T, T_do, TT, i)
    torch.cuda.synchronize()
    sol.close()
    host = lambda t: None if t is None else t.cpu().numpy()
    return host(s), host(u), host(b), float(T_do.cpu()[0]), float(TT.cpu()[0])


@pytest.mark.parametrize("physics", [g.EULER, g.MHD])
@pytest.mark.parametrize("mode", [g.MODE_FAST, g.MODE_PARITY])
def test_cpp_client_equals_python_driver(cuda, tmp_path, physics, mode):
    exe = build_client(tmp_path)
    N, M = 64, 48
    if physics == g.EULER:
        cfg, s, u, b = problems.kelvin_helmholtz(N, M, mode=mode)
    else:
        cfg, s, u, b = problems.orszag_tang(N, M, mode=mode)
    parts = [s, u] + ([] if b is None else [b])
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    np.concatenate([np.ascontiguousarray(p).ravel() for p in parts]).astype("<f8").tofile(inp)
    r = subprocess.run([exe, str(physics), str(mode), str(N), str(M), str(ITERS), str(inp),
                        str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype="<f8")
    K = N * M
    cs, cu = got[:2 * K].reshape(K, 2), got[2 * K:4 * K].reshape(K, 2)
    cb = got[4 * K:7 * K].reshape(K, 3) if b is not None else None
    c_Tdo, c_TT = got[-2], got[-1]
    ps, pu, pb, p_Tdo, p_TT = python_loop(cfg, s, u, b)
    assert np.array_equal(cs, ps) and np.array_equal(cu, pu)
    if b is not None:
        assert np.array_equal(cb, pb)
    assert c_Tdo == p_Tdo and c_TT == p_TT
