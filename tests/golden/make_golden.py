"""Writes the golden vectors in this directory from the reference's OWN code.

The reference (Gas_Dinamic.cu, kernel.cu) is compiled for the host by oracle/ref_build
(``make -C oracle ref REF=<checkout>``) into oracle/_ref/libgdref.so; this script calls
its functions and stores inputs and outputs as .npz fixtures.  The reference sources are
needed only to regenerate the fixtures (GD_REFERENCE_SRC names the checkout); the tests
read the committed .npz files.

    GD_REFERENCE_SRC=<reference checkout> python tests/golden/make_golden.py

Fixtures:
  faces_hllc.npz   Euler HLLC_Aleksashov (kernel.cu:853) on random and branch-targeted states
  faces_hlld.npz   HLLDQ_Korolkov (Gas_Dinamic.cu:964), metod 3 (HLLD) and 2 (HLLC-MHD)
  recon.npz        minmod / linear / linear2 (kernel.cu:51-84)
  step_native.npz  one step of Kernel_TVD (metod 3, 2), add2 (metod 2, 3), Ker_Dekard on
                   small random grids with the reference's own boundary conditions
  run_native.npz   20 steps of the reference protocol (Kernel_TVD + funk_time) from the
                   reference's wind initial condition on a reduced axisymmetric grid
  faces_hll.npz    Euler HLL (kernel.cu:1485) on random and branch-targeted faces, and one
                   Ker_Dekard step with method 0 (HLL everywhere)
  gkr.npz          Kernel_GKR (kernel.cu:2663-3284, the MUSCL-Hancock step): one step on
                   random states of six small grids whose sizes reach every edge branch of
                   its stencil, and 20 steps of Kernel_GKR + funk_time from the wind of
                   problems.hancock_wind on a reduced grid
  io_files.npz     the reference's state files for one random state with hard-to-print
                   values: print_file_mini / print_file_mini2 (both overloads) Tecplot
                   snapshots (kernel.cu:3682-3808) and the restart dump of its main loop
                   (kernel.cu:4245-4254), as bytes

    python tests/golden/make_golden.py [fixture ...]   (default: all)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from golikov_2d_gb300 import problems  # noqa: E402

SEED = 20261203
NORMALS = np.array([[1.0, 0.0], [0.0, -1.0], [-1.0, 0.0], [0.0, 1.0]])


def euler_states(rng, n):
    L = np.stack([rng.uniform(0.05, 3.0, n), rng.uniform(0.02, 3.0, n),
                  rng.uniform(-3, 3, n), rng.uniform(-3, 3, n)], 1)
    R = np.stack([rng.uniform(0.05, 3.0, n), rng.uniform(0.02, 3.0, n),
                  rng.uniform(-3, 3, n), rng.uniform(-3, 3, n)], 1)
    k = n // 8
    R[:k] = L[:k]                                    # identical states, F(U,U) = F(U)
    L[k:2 * k, 2] = 6.0 + rng.uniform(0, 2, k)       # supersonic to the right (SL > 0)
    R[k:2 * k, 2] = 6.0 + rng.uniform(0, 2, k)
    L[2 * k:3 * k, 2] = -6.0 - rng.uniform(0, 2, k)  # supersonic to the left (SR < 0)
    R[2 * k:3 * k, 2] = -6.0 - rng.uniform(0, 2, k)
    R[3 * k:4 * k, 1] = L[3 * k:4 * k, 1] * 1e-4     # strong pressure jumps
    R[4 * k:5 * k, 0] = L[4 * k:5 * k, 0] * 1e-3     # strong density jumps
    # mirror-symmetric pairs: SM == 0 exactly
    R[5 * k:6 * k] = L[5 * k:6 * k]
    R[5 * k:6 * k, 2] = -L[5 * k:6 * k, 2]
    return L, R


def mhd_states(rng, n):
    def side():
        return np.stack([rng.uniform(0.05, 3.0, n), rng.uniform(0.02, 3.0, n),
                         rng.uniform(-3, 3, n), rng.uniform(-3, 3, n), np.zeros(n),
                         rng.uniform(-4, 4, n), rng.uniform(-4, 4, n), rng.uniform(-4, 4, n)], 1)
    L, R = side(), side()
    k = n // 10
    R[:k] = L[:k]
    L[k:2 * k, 5:8] = 0.0                      # no field at all
    R[k:2 * k, 5:8] = 0.0
    L[2 * k:3 * k, 5] = 0.0                    # Bn = 0: idbn = 0 branch
    R[2 * k:3 * k, 5] = 0.0
    L[2 * k:3 * k, 6] = 0.0
    R[2 * k:3 * k, 6] = 0.0
    L[3 * k:4 * k, 5] = 1e-7                   # |bn| below 1e-6
    R[3 * k:4 * k, 5] = -1e-7
    L[3 * k:4 * k, 6] = 1e-7
    R[3 * k:4 * k, 6] = -1e-7
    L[4 * k:5 * k, 2:4] = 8.0 + rng.uniform(0, 2, (k, 2))   # supersonic
    R[4 * k:5 * k, 2:4] = 8.0 + rng.uniform(0, 2, (k, 2))
    L[5 * k:6 * k, 2:4] = -8.0 - rng.uniform(0, 2, (k, 2))
    R[5 * k:6 * k, 2:4] = -8.0 - rng.uniform(0, 2, (k, 2))
    # strong normal field, weak tangential field: star-state degeneracy (tt ~ 0)
    L[6 * k:7 * k, 5:7] = np.stack([rng.uniform(3, 6, k), 1e-6 * rng.uniform(-1, 1, k)], 1)
    R[6 * k:7 * k, 5:7] = np.stack([L[6 * k:7 * k, 5], 1e-6 * rng.uniform(-1, 1, k)], 1)
    L[6 * k:7 * k, 7] = 0.0
    R[6 * k:7 * k, 7] = 0.0
    return L, R


def faces(ref):
    rng = np.random.default_rng(SEED)
    out = {}
    n = 1600
    L, R = euler_states(rng, n)
    nrm = NORMALS[rng.integers(0, 4, n)]
    gam = np.where(rng.uniform(size=n) < 0.5, 1.4, 5.0 / 3.0)
    T = np.zeros(n)
    F = np.zeros((n, 4))
    for i in range(n):
        ref.set_params(gam[i], 0.4, 64, 64, 1.0, 1.0)
        T[i], F[i] = ref.hllc(L[i], R[i], nrm[i, 0], nrm[i, 1], 1.0 / 128)
    np.savez_compressed(os.path.join(HERE, "faces_hllc.npz"), L=L, R=R, normal=nrm, gamma=gam,
                        krit=0.4, rad=1.0 / 128, t=T, flux=F)
    n = 2400
    L, R = mhd_states(rng, n)
    nrm = NORMALS[rng.integers(0, 4, n)]
    meth = np.where(np.arange(n) % 3 == 0, 2, 3)
    T = np.zeros(n)
    F = np.zeros((n, 8))
    ref.set_params(5.0 / 3.0, 0.4, 64, 64, 1.0, 1.0)
    for i in range(n):
        T[i], F[i] = ref.hlld(L[i], R[i], nrm[i, 0], nrm[i, 1], 0.0, 1.0 / 128, int(meth[i]))
    np.savez_compressed(os.path.join(HERE, "faces_hlld.npz"), L=L, R=R, normal=nrm,
                        method=meth, gamma=5.0 / 3.0, krit=0.4, rad=1.0 / 128, t=T, flux=F)


def recon(ref):
    rng = np.random.default_rng(SEED + 1)
    n = 1000
    a = rng.uniform(-1, 1, (n, 2))
    a[: n // 6, 1] = 0.0
    a[n // 6: n // 3, 1] = a[n // 6: n // 3, 0]
    mm = np.array([ref.lib.gdref_minmod(x, y) for x, y in a])
    x = rng.uniform(0.0, 5.0, n)
    h = rng.uniform(1e-4, 1e-1, n)
    t = rng.uniform(-2, 2, (n, 3))
    lin = np.array([ref.lib.gdref_linear(x[i], t[i, 0], x[i] + h[i], t[i, 1], x[i] + 2.0 * h[i],
                                         t[i, 2], x[i] + h[i] / 2.0) for i in range(n)])
    A = np.zeros(n)
    B = np.zeros(n)
    import ctypes
    for i in range(n):
        pa, pb = ctypes.c_double(), ctypes.c_double()
        ref.lib.gdref_linear2(x[i] - h[i], t[i, 0], x[i], t[i, 1], x[i] + h[i], t[i, 2],
                              x[i] - h[i] / 2.0, x[i] + h[i] / 2.0, ctypes.byref(pa),
                              ctypes.byref(pb))
        A[i], B[i] = pa.value, pb.value
    np.savez_compressed(os.path.join(HERE, "recon.npz"), mm_in=a, mm=mm, x=x, h=h, t=t, lin=lin,
                        A=A, B=B)


def random_state(rng, K):
    s = np.stack([rng.uniform(0.3, 2.0, K), rng.uniform(0.1, 2.0, K)], 1)
    u = rng.uniform(-1.0, 1.0, (K, 2))
    b = rng.uniform(-2.0, 2.0, (K, 3))
    return s, u, b


def step_native(ref):
    rng = np.random.default_rng(SEED + 2)
    N, M, xmax, ymax = 40, 24, 9.0, 5.0
    K = N * M
    s, u, b = random_state(rng, K)
    T_do = 2e-3
    out = dict(N=N, M=M, xmax=xmax, ymax=ymax, s=s, u=u, b=b, T_do=T_do)
    g = 5.0 / 3.0
    ref.set_params(g, 0.25, N, M, xmax, ymax)
    for meth in (3, 2):
        s2, u2, b2, T = ref.kernel_tvd(s, u, b, T_do, 0, meth)
        out.update({f"tvd{meth}_s": s2, f"tvd{meth}_u": u2, f"tvd{meth}_b": b2, f"tvd{meth}_T": T})
        s2, u2, b2, T = ref.add2(s, u, b, T_do, 0, meth)
        out.update({f"add{meth}_s": s2, f"add{meth}_u": u2, f"add{meth}_b": b2, f"add{meth}_T": T})
    ref.set_params(1.4, 0.4, N, M, xmax, ymax)
    s2, u2, T = ref.ker_dekard(s, u, T_do)
    out.update({"dek_s": s2, "dek_u": u2, "dek_T": T})
    np.savez_compressed(os.path.join(HERE, "step_native.npz"), **out)


def run_native(ref, nsteps=20):
    N, M, xmax, ymax = 64, 36, 2.25, 1.25
    cfg, s, u, b = problems.stellar_wind(N, M, xmax, ymax)
    ref.set_params(cfg.gamma, cfg.krit, N, M, xmax, ymax)
    T_do, TT = 1e-8, 0.0
    s0, u0, b0 = s.copy(), u.copy(), b.copy()
    for _ in range(nsteps):
        s, u, b, T = ref.kernel_tvd(s, u, b, T_do, 0, 3)
        T_do = T
        TT += T_do
    np.savez_compressed(os.path.join(HERE, "run_native.npz"), N=N, M=M, xmax=xmax, ymax=ymax,
                        nsteps=nsteps, s0=s0, u0=u0, b0=b0, s=s, u=u, b=b, T_do=T_do, TT=TT)


def hll_golden(ref):
    """HLL (kernel.cu:1485-1609) on random and branch-targeted faces, plus one Ker_Dekard step
    with method 0 (HLL everywhere, kernel.cu:1796-1802)."""
    rng = np.random.default_rng(SEED + 11)
    n = 1600
    L, R = euler_states(rng, n)
    k = n // 8
    L[6 * k:6 * k + k // 2, 0] = 0.0                  # rho <= 0: sound speed 0
    R[6 * k + k // 2:7 * k, 0] = -rng.uniform(0, 1, k - k // 2)
    L[7 * k:, 2] = R[7 * k:, 2]                       # equal normal speeds (ties in min/max)
    nrm = NORMALS[rng.integers(0, 4, n)]
    gam = np.where(rng.uniform(size=n) < 0.5, 1.4, 5.0 / 3.0)
    T = np.zeros(n)
    F = np.zeros((n, 4))
    for i in range(n):
        ref.set_params(gam[i], 0.4, 64, 64, 1.0, 1.0)
        T[i], F[i] = ref.hll(L[i], R[i], nrm[i, 0], nrm[i, 1], 1.0 / 128)
    N, M, xmax, ymax = 40, 24, 9.0, 5.0
    s, u, _ = random_state(rng, N * M)
    T_do = 2e-3
    ref.set_params(1.4, 0.4, N, M, xmax, ymax)
    s2, u2, T1 = ref.ker_dekard(s, u, T_do, method=0)
    np.savez_compressed(os.path.join(HERE, "faces_hll.npz"), L=L, R=R, normal=nrm, gamma=gam,
                        krit=0.4, rad=1.0 / 128, t=T, flux=F, N=N, M=M, xmax=xmax, ymax=ymax,
                        s=s, u=u, T_do=T_do, dek_s=s2, dek_u=u2, dek_T=T1)


def io_state(rng, K):
    """A state whose numbers exercise every branch of %g: magnitudes 1e-8..1e3, negative
    and zero densities (the Tecplot writer's rho > 0 branch), signed zeros, exact decimal
    ties, powers of ten and their neighbours, subnormals and extremes."""
    s = np.stack([10 ** rng.uniform(-8, 3, K) * np.where(rng.random(K) < 0.05, -1, 1),
                  10 ** rng.uniform(-8, 3, K)], 1)
    u = rng.standard_normal((K, 2)) * 10 ** rng.uniform(-5, 2, (K, 2))
    b = rng.standard_normal((K, 3)) * 10 ** rng.uniform(-5, 2, (K, 3))
    special = [0.0, -0.0, 1234565.0, 1234575.0, 0.5, 2.5e-5, 99999.95, 999999.5, 9.9999995,
               1e-5, 1e-4, 1e5, 1e6, 1e-300, 5e-324, 2.2250738585072014e-308,
               1.7976931348623157e308, -123456.5, 0.1, 1.0 / 3.0, 1e21, 1e22, 1e23,
               np.nextafter(1e-4, 0), np.nextafter(1e6, 2e6), 100000.5]
    flat = np.concatenate([s.ravel(), u.ravel(), b.ravel()])
    idx = rng.choice(flat.size, len(special), replace=False)
    flat[idx] = special
    s = flat[:2 * K].reshape(K, 2)
    u = flat[2 * K:4 * K].reshape(K, 2)
    b = flat[4 * K:].reshape(K, 3)
    s[3, 0] = 0.0
    return s, u, b


def io_files(ref):
    N, M, xmax, ymax, gamma = 23, 17, 9.0, 5.0, 5.0 / 3.0
    rng = np.random.default_rng(SEED + 7)
    s, u, b = io_state(rng, N * M)
    ref.set_params(gamma, 0.25, N, M, xmax, ymax)
    out = {}
    tmp = os.path.join(HERE, "_io_tmp.dat")
    for name, call in (("tec_euler", lambda: ref.print_tecplot(s, u, None, 0, 0.0, tmp)),
                       ("tec_mhd", lambda: ref.print_tecplot(s, u, b, 1, 0.0, tmp)),
                       ("tec_mhd_t", lambda: ref.print_tecplot(s, u, b, 2, 0.123456789, tmp)),
                       ("restart", lambda: ref.write_restart(s, u, b, tmp))):
        call()
        with open(tmp, "rb") as f:
            out[name] = np.frombuffer(f.read(), np.uint8)
    os.remove(tmp)
    np.savez_compressed(os.path.join(HERE, "io_files.npz"), N=N, M=M, xmax=xmax, ymax=ymax,
                        gamma=gamma, nmin=3, ttt=0.123456789, s=s, u=u, b=b, **out)


GKR_CASES = ((40, 24, 9.0, 5.0), (33, 17, 9.0, 5.0), (24, 16, 30.0, 20.0), (7, 5, 9.0, 5.0),
             (3, 3, 9.0, 5.0), (4, 6, 9.0, 5.0))


def gkr_golden(ref, nsteps=20):
    rng = np.random.default_rng(SEED + 13)
    T_do = 2e-3
    out = dict(ncases=len(GKR_CASES), T_do=T_do, gamma=5.0 / 3.0, krit=0.25)
    for c, (N, M, xmax, ymax) in enumerate(GKR_CASES):
        s, u, b = random_state(rng, N * M)
        ref.set_params(5.0 / 3.0, 0.25, N, M, xmax, ymax)
        s2, u2, b2, T = ref.kernel_gkr(s, u, b, T_do, 0, 3)
        out.update({f"c{c}_NM": np.array([N, M]), f"c{c}_ext": np.array([xmax, ymax]),
                    f"c{c}_s": s, f"c{c}_u": u, f"c{c}_b": b,
                    f"c{c}_s2": s2, f"c{c}_u2": u2, f"c{c}_b2": b2, f"c{c}_T": T})
    N, M, xmax, ymax = 72, 40, 9.0, 5.0
    cfg, s, u, b = problems.hancock_wind(N, M, xmax, ymax)
    ref.set_params(cfg.gamma, cfg.krit, N, M, xmax, ymax)
    out.update(run_N=N, run_M=M, run_ext=np.array([xmax, ymax]), run_nsteps=nsteps,
               run_s0=s.copy(), run_u0=u.copy(), run_b0=b.copy())
    T_do, TT = 1e-8, 0.0
    for _ in range(nsteps):
        s, u, b, T = ref.kernel_gkr(s, u, b, T_do, 0, 3)
        T_do = T
        TT += T_do
    out.update(run_s=s, run_u=u, run_b=b, run_T_do=T_do, run_TT=TT)
    np.savez_compressed(os.path.join(HERE, "gkr.npz"), **out)


def main():
    oracle.build(ref=True)
    ref = oracle.Reference()
    ref.lib.gdref_set_threads(1)
    jobs = {"faces": faces, "recon": recon, "step_native": step_native,
            "run_native": run_native, "io_files": io_files, "hll": hll_golden,
            "gkr": gkr_golden}
    for name in (sys.argv[1:] or list(jobs)):
        jobs[name](ref)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
