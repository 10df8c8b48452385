"""Host logic of the CG's coarse correction, without a GPU: the band Cholesky inverse of the coarse operator
(ikr_ls_s::band_spd_inverse in ikarus_gb300/csrc/host_internal.h), compiled from tests/cpp/band_inverse.cpp.
A random SPD block-tridiagonal matrix of 6x6 blocks with one aggregate without stiffness and one repeated mode:
the inverse is exact on the kept modes, zero on the seven dropped ones, and symmetric."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_band_inverse_of_the_coarse_operator(tmp_path):
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "band_inverse")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + inc, os.path.join(ROOT, "tests", "cpp", "band_inverse.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True, timeout=60).stdout.split()
    err, dropped_max, asym, dropped = float(out[0]), float(out[1]), float(out[2]), int(out[3])
    assert err <= 1e-12
    assert dropped_max == 0.0 and asym == 0.0
    assert dropped == 7


# ---- the coarse correction's algorithm restated in numpy on the oracle's FP64 tangent (no GPU) ----
# Slabs of equal node count along the longest axis, six rigid-body modes each about the slab centroid, zero at
# constrained dofs (ikr_ls_s::coarse_layout); A_c by probing: for every colour c of the slab chain coloured
# mod 2 reach + 1, K times the sum of the colour's mode columns, restricted to every slab and placed at the one
# slab of that colour within reach (ikr_ls_s::coarse_operator, coarse_probe_kernel, coarse_galerkin_kernel).

def _two_level_setup(p, n_slabs):
    import numpy as np
    import scipy.sparse as sp

    import oracle
    o = oracle.from_problem(p)
    cp, ri, va, n = o.assemble_matrix_csc(np.zeros(p.n_dofs), 0.1)
    K = sp.csc_matrix((va, ri, cp), shape=(n, n)).tocsr()
    b = -o.assemble_vector(np.zeros(p.n_dofs), 0.1)
    X = p.mesh.coords
    nn = len(X)
    ax = int(np.argmax(X.max(0) - X.min(0)))
    order = np.argsort(X[:, ax], kind="stable")
    agg = np.empty(nn, dtype=int)
    agg[order] = np.arange(nn) * n_slabs // nn
    cen = np.array([X[agg == a].mean(0) for a in range(n_slabs)])
    y = (X - cen[agg]).astype(np.float32).astype(np.float64)
    free = 1 - p.fixed.reshape(nn, 3)
    cols = np.zeros((nn, 3, 6))
    cols[:, 0, 0] = cols[:, 1, 1] = cols[:, 2, 2] = 1.0
    cols[:, 0, 4], cols[:, 0, 5] = y[:, 2], -y[:, 1]
    cols[:, 1, 3], cols[:, 1, 5] = -y[:, 2], y[:, 0]
    cols[:, 2, 3], cols[:, 2, 4] = y[:, 1], -y[:, 0]
    cols *= free[:, :, None]
    rows = np.repeat(np.arange(n), 6)
    colidx = (6 * np.repeat(agg, 3)[:, None] + np.arange(6)).ravel()
    P = sp.csr_matrix((cols.reshape(n, 6).ravel(), (rows, colidx)), shape=(n, 6 * n_slabs))
    return K, b, P, agg, cols


def _probed_coarse_operator(K, agg, cols, n_slabs):
    import numpy as np
    Kc = K.tocoo()
    reach = int(np.abs(agg[Kc.row // 3] - agg[Kc.col // 3]).max())
    ncol = min(2 * reach + 1, n_slabs)
    nn = len(agg)
    Ac = np.zeros((6 * n_slabs, 6 * n_slabs))
    for c in range(ncol):
        on = (agg % ncol == c)[:, None, None]
        V = (cols * on).transpose(2, 0, 1).reshape(6, 3 * nn)
        W = np.array([K @ V[m] for m in range(6)]).reshape(6, nn, 3)
        contrib = np.einsum("icr,mic->irm", cols, W)  # per node: P_i^T (K V_m)_i
        for s in range(n_slabs):
            near = [s + d for d in range(-reach, reach + 1) if 0 <= s + d < n_slabs and (s + d) % ncol == c]
            if near:
                Ac[6 * s:6 * s + 6, 6 * near[0]:6 * near[0] + 6] = contrib[agg == s].sum(0)
    return 0.5 * (Ac + Ac.T), reach


def test_probed_coarse_operator_is_the_galerkin_product():
    import numpy as np

    from ikarus_gb300 import problems
    p = problems.cantilever(32, 4, 4, jitter=0.1, seed=3)
    K, b, P, agg, cols = _two_level_setup(p, 8)
    Ac, reach = _probed_coarse_operator(K, agg, cols, 8)
    exact = (P.T @ K @ P).toarray()
    assert reach == 1
    assert np.abs(Ac - exact).max() <= 1e-12 * np.abs(exact).max()


def test_two_level_preconditioner_cuts_cg_iterations():
    """Same solution, several times fewer iterations than block Jacobi alone on a slender cantilever."""
    import numpy as np

    from ikarus_gb300 import problems
    p = problems.cantilever(32, 4, 4, jitter=0.1, seed=3)
    K, b, P, agg, cols = _two_level_setup(p, 8)
    nn = len(agg)
    idx = np.arange(nn)
    D = np.stack([np.stack([K[3 * idx + r, 3 * idx + c].A1 for c in range(3)], -1) for r in range(3)], 1)
    Dinv = np.linalg.inv(D)
    Ac_inv = np.linalg.inv((P.T @ K @ P).toarray())

    def pcg(prec, rtol=1e-8):
        x, r = np.zeros_like(b), b.copy()
        z = prec(r)
        d, rz = z.copy(), r @ z
        for it in range(1, 20000):
            q = K @ d
            a = rz / (d @ q)
            x += a * d
            r -= a * q
            if np.linalg.norm(r) <= rtol * np.linalg.norm(b):
                return x, it
            z = prec(r)
            rz, rz0 = r @ z, rz
            d = z + rz / rz0 * d
        raise AssertionError("no convergence")

    def bj(r):
        return np.einsum("nij,nj->ni", Dinv, r.reshape(nn, 3)).ravel()

    x0, it0 = pcg(bj)
    x1, it1 = pcg(lambda r: bj(r) + P @ (Ac_inv @ (P.T @ r)))
    assert np.abs(x1 - x0).max() <= 1e-6 * np.abs(x0).max()
    assert it1 * 3 < it0, (it0, it1)
