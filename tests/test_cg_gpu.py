"""GPU parity of the CG path through the C ABI against the oracle (CPU
restatement of the reference's CG, conjugateGradient/cg_cpu.cpp:40-81).

CG on the GPU reduces dot products in a different order than the sequential
CPU loop, so results are not bit-identical; the bar is the FP64 CG
contract: the same iteration count (within 1, or 1% for long solves) and a true
relative residual ||b - A x|| / ||b|| <= 1e-10 recomputed in FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def true_rel(rp, ci, v, b, x):
    from oracle import oracle as O
    r = b - O.spmv_csr(rp, ci, np.asarray(v, np.float64), np.asarray(x, np.float64))
    return np.linalg.norm(r) / np.linalg.norm(b)


def it_close(a, b):
    return abs(a - b) <= max(1, int(0.01 * max(a, b)))


@pytest.mark.parametrize("kernel", ["persistent", "per_step"])
@pytest.mark.parametrize("matrix", ["lap2d", "lap3d", "spd"])
def test_cg_fp64_csr_vs_oracle(native, cuda, oracle, kernel, matrix):
    from perks_gb300 import matrices as M
    rp, ci, v = {"lap2d": lambda: M.laplacian_2d(96), "lap3d": lambda: M.laplacian_3d(24),
                 "spd": lambda: M.random_spd(20000, 3)}[matrix]()
    b = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    xo, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=20000, stop=1, tol=1e-10)
    x, res = native.cg_csr(rp, ci, v, b, dtype="fp64", tol=1e-10, kernel=kernel, device=cuda)
    assert it_close(res["iterations"], it), (res, it)
    assert res["true_rel_res"] <= 1e-10 * 1.05
    assert true_rel(rp, ci, v, b, x.cpu().numpy()) <= 1e-10 * 1.05
    assert np.allclose(x.cpu().numpy(), xo, rtol=1e-7, atol=1e-9)


def test_cg_dia_matches_csr(native, cuda, oracle):
    from perks_gb300 import matrices as M
    rp, ci, v = M.laplacian_2d(80)
    off, data = M.csr_to_dia(rp, ci, v)
    b = np.random.default_rng(2).uniform(-1, 1, len(rp) - 1)
    xo, it, _ = oracle.cg_dia(off, data, b, max_iter=20000, stop=1, tol=1e-10)
    x, res = native.cg_dia(off, data, b, dtype="fp64", tol=1e-10, device=cuda)
    assert it_close(res["iterations"], it)
    assert true_rel(rp, ci, v, b, x.cpu().numpy()) <= 1e-10 * 1.05


def test_cg_reference_mode_tridiag(native, cuda, oracle):
    """The reference's own setting: genTridiag matrix, rhs = 1, x0 = 0, stop on
    absolute r.r < tol^2 (conjugateGradient/cg_driver.cu:140-210)."""
    for n in (1000, 100000):
        rp, ci, v = oracle.gen_tridiag(n, 1, np.float64)
        b = np.ones(n)
        xo, it, rr, _ = oracle.cg(rp, ci, v, b, max_iter=n, stop=0, tol=1e-10)
        x, res = native.cg_csr(rp, ci, v, b, dtype="fp64", stop="abs", tol=1e-10, max_iter=n, device=cuda)
        assert it_close(res["iterations"], it), (n, res, it)
        assert res["rr"] < 1e-20
        assert np.allclose(x.cpu().numpy(), xo, rtol=1e-8, atol=1e-10)


def test_cg_float_build_tracks_oracle(native, cuda, oracle):
    """FP32 (the reference's float build): a few iterations agree with the
    float oracle to float rounding."""
    rp, ci, v = oracle.gen_tridiag(5000, 2, np.float32)
    b = np.ones(5000, np.float32)
    xo, it, _, tr = oracle.cg(rp, ci, v, b, max_iter=6, static_iter=True, trace=True)
    x, res = native.cg_csr(rp, ci, v, b, dtype="fp32", max_iter=6, static_iter=True, device=cuda)
    assert res["iterations"] == 6
    assert np.allclose(x.cpu().numpy(), xo, rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("matrix", ["lap2d", "spd"])
@pytest.mark.parametrize("fmt", ["csr", "dia"])
def test_cg_mixed_reaches_fp64_accuracy(native, cuda, oracle, matrix, fmt):
    from perks_gb300 import matrices as M
    if matrix == "spd" and fmt == "dia":
        pytest.skip("random pattern has too many diagonals for DIA")
    rp, ci, v = M.laplacian_2d(128) if matrix == "lap2d" else M.random_spd(50000, 4)
    b = np.random.default_rng(3).uniform(-1, 1, len(rp) - 1)
    _, it64, _, _ = oracle.cg(rp, ci, v, b, max_iter=50000, stop=1, tol=1e-10)
    if fmt == "csr":
        x, res = native.cg_csr(rp, ci, v, b, dtype="mixed", tol=1e-10, device=cuda)
    else:
        off, data = M.csr_to_dia(rp, ci, v)
        x, res = native.cg_dia(off, data, b, dtype="mixed", tol=1e-10, device=cuda)
    assert true_rel(rp, ci, v, b, x.cpu().numpy()) <= 1e-10 * 1.05
    assert res["outer"] >= 1
    assert res["iterations"] <= 2 * it64 + 50, (res, it64)


def test_cg_breakdown_reported(native, cuda):
    from perks_gb300 import matrices as M
    rp, ci, v = M.laplacian_2d(16)
    b = np.ones(len(rp) - 1)
    x, res = native.cg_csr(rp, ci, -v, b, dtype="fp64", device=cuda, check=False)
    assert res["status"] == -17


def test_cg_not_converged_reported(native, cuda):
    from perks_gb300 import matrices as M
    rp, ci, v = M.laplacian_2d(64)
    b = np.ones(len(rp) - 1)
    x, res = native.cg_csr(rp, ci, v, b, dtype="fp64", max_iter=5, device=cuda, check=False)
    assert res["status"] == -18 and res["iterations"] == 5


def test_spmv_matches_oracle(native, cuda, oracle):
    from perks_gb300 import matrices as M
    rp, ci, v = M.random_spd(30000, 5)
    x = np.random.default_rng(4).standard_normal(len(rp) - 1)
    y = native.spmv_csr(rp, ci, v, x, device=cuda).cpu().numpy()
    assert np.allclose(y, oracle.spmv_csr(rp, ci, v, x), rtol=1e-13, atol=1e-12)
    rp, ci, v = M.laplacian_3d(20)
    off, data = M.csr_to_dia(rp, ci, v)
    x = np.random.default_rng(5).standard_normal(len(rp) - 1)
    y = native.spmv_dia(off, data, x, device=cuda).cpu().numpy()
    assert np.allclose(y, oracle.spmv_dia(off, data, x), rtol=1e-13, atol=1e-12)


def _permuted(rp, ci, v, seed):
    """P A P^T for a random permutation, columns sorted within rows."""
    import scipy.sparse as sp
    n = len(rp) - 1
    A = sp.csr_matrix((v, ci, rp), shape=(n, n))
    perm = np.random.default_rng(seed).permutation(n)
    B = A[perm][:, perm].tocsr()
    B.sort_indices()
    return B.indptr.astype(np.int32), B.indices.astype(np.int32), B.data


def _shuffled_columns(rp, ci, v, seed):
    """The same matrix with each row's entries in a random order."""
    rng = np.random.default_rng(seed)
    ci2, v2 = ci.copy(), v.copy()
    for i in range(len(rp) - 1):
        a, b = rp[i], rp[i + 1]
        o = rng.permutation(b - a) + a
        ci2[a:b], v2[a:b] = ci[o], v[o]
    return rp, ci2, v2


def _arrow(n, seed):
    """Arrowhead SPD matrix: a tridiagonal band plus a dense first row and
    column (row 0 holds n entries), diagonally dominant."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    off = rng.uniform(-1, 0, n - 1)
    arm = rng.uniform(-1, 1, n - 1) * 0.01
    A = sp.diags([off, off], [-1, 1], shape=(n, n)).tolil()
    A[0, 1:] = arm
    A[1:, 0] = arm[:, None]
    A = A.tocsr()
    d = np.abs(A).sum(axis=1).A1 + rng.uniform(0.1, 1.0, n)
    A = (A + sp.diags(d)).tocsr()
    A.sort_indices()
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data


# CSR layouts the persistent solver chooses internally (perks_cg_result
# .layout): diagonal structure (sorted columns, few diagonals: DIA copy, 1),
# bounded rows on scattered diagonals (ELL copy, 2), unsorted columns (ELL:
# the DIA copy needs sorted columns), irregular rows of 3..60 entries (SELL
# copy, 3), and one dense row among short ones (SELL padding too large: CSR
# as given, lane groups, 0).
@pytest.mark.parametrize("layout,expect", [("diagonals", 1), ("scattered", 2), ("unsorted", 2), ("irregular", 3),
                                           ("arrow", 0)])
@pytest.mark.parametrize("dtype", ["fp64", "mixed", "fp32"])
def test_cg_csr_layouts(native, cuda, oracle, layout, expect, dtype):
    pytest.importorskip("scipy")
    from perks_gb300 import matrices as M
    base = M.laplacian_2d(96)
    rp, ci, v = {"diagonals": lambda: base, "scattered": lambda: _permuted(*base, seed=3),
                 "unsorted": lambda: _shuffled_columns(*base, seed=4),
                 "irregular": lambda: M.random_spd(20000, 5), "arrow": lambda: _arrow(20000, 6)}[layout]()
    b = np.random.default_rng(6).uniform(-1, 1, len(rp) - 1)
    _, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=20000, stop=1, tol=1e-10)
    if dtype == "fp32":
        # the reference's float build: tracks the float oracle for a few iterations
        v32, b32 = v.astype(np.float32), b.astype(np.float32)
        xo, _, _, _ = oracle.cg(rp, ci, v32, b32, max_iter=8, static_iter=True)
        x, res = native.cg_csr(rp, ci, v32, b32, dtype="fp32", max_iter=8, static_iter=True, device=cuda)
        assert res["layout"] == expect
        # normwise: the arrow's dense row sums 20000 FP32 terms with
        # cancellation, in another order than the sequential oracle
        xg = x.cpu().numpy().astype(np.float64)
        assert np.linalg.norm(xg - xo) <= 1e-4 * np.linalg.norm(xo)
        return
    x, res = native.cg_csr(rp, ci, v, b, dtype=dtype, tol=1e-10, device=cuda)
    assert res["layout"] == expect, res
    if dtype == "fp64":
        assert it_close(res["iterations"], it), (layout, res, it)
    assert res["true_rel_res"] <= 1e-10 * 1.05
    assert true_rel(rp, ci, v, b, x.cpu().numpy()) <= 1e-10 * 1.05


@pytest.mark.parametrize("cluster", [2, 4, 8])
@pytest.mark.parametrize("matrix,dtype", [("lap2d", "fp64"), ("spd", "fp64"), ("lap2d", "mixed"), ("spd", "fp32")])
def test_cg_cluster_combine(native, cuda, oracle, cluster, matrix, dtype):
    """Grid reductions through thread-block clusters (partials combined over
    distributed shared memory, one grid-barrier arrival per cluster): the
    same convergence as the oracle, whole clusters, and the same result on a
    second run (the combine order is fixed)."""
    from perks_gb300 import matrices as M
    rp, ci, v = M.laplacian_2d(96) if matrix == "lap2d" else M.random_spd(20000, 3)
    b = np.random.default_rng(8).uniform(-1, 1, len(rp) - 1)
    if dtype == "fp32":
        v32, b32 = v.astype(np.float32), b.astype(np.float32)
        xo, _, _, _ = oracle.cg(rp, ci, v32, b32, max_iter=10, static_iter=True)
        xs = [native.cg_csr(rp, ci, v32, b32, dtype="fp32", max_iter=10, static_iter=True, cluster=cluster,
                            device=cuda) for _ in range(2)]
        assert xs[0][1]["ctas"] % cluster == 0
        assert np.array_equal(xs[0][0].cpu().numpy(), xs[1][0].cpu().numpy())
        xg = xs[0][0].cpu().numpy().astype(np.float64)
        assert np.linalg.norm(xg - xo) <= 1e-4 * np.linalg.norm(xo)
        return
    _, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=20000, stop=1, tol=1e-10)
    runs = [native.cg_csr(rp, ci, v, b, dtype=dtype, tol=1e-10, cluster=cluster, device=cuda) for _ in range(2)]
    (x, res), (x2, res2) = runs
    assert res["ctas"] % cluster == 0 and res["ctas"] >= cluster
    assert np.array_equal(x.cpu().numpy(), x2.cpu().numpy()) and res["iterations"] == res2["iterations"]
    if dtype == "fp64":
        assert it_close(res["iterations"], it), (res, it)
    assert true_rel(rp, ci, v, b, x.cpu().numpy()) <= 1e-10 * 1.05


@pytest.mark.parametrize("matrix", ["lap2d", "lap3d", "spd", "tridiag"])
@pytest.mark.parametrize("fmt", ["csr", "dia"])
def test_cg_single_reduction_vs_oracle(native, cuda, oracle, matrix, fmt):
    """Single-reduction CG (Chronopoulos & Gear): the same iteration count as
    the FP64 oracle's plain CG (within 1, or 1% for long solves), a true
    residual below the tolerance recomputed on the host, and the same result
    on a second run."""
    from perks_gb300 import matrices as M
    if matrix == "spd" and fmt == "dia":
        pytest.skip("random pattern has too many diagonals for DIA")
    rp, ci, v = {"lap2d": lambda: M.laplacian_2d(96), "lap3d": lambda: M.laplacian_3d(24),
                 "spd": lambda: M.random_spd(20000, 3),
                 "tridiag": lambda: oracle.gen_tridiag(20000, 1, np.float64)}[matrix]()
    b = np.random.default_rng(9).uniform(-1, 1, len(rp) - 1)
    _, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=20000, stop=1, tol=1e-10)
    runs = []
    for _ in range(2):
        if fmt == "csr":
            runs.append(native.cg_csr(rp, ci, v, b, dtype="fp64", tol=1e-10, algorithm="single_reduction",
                                      device=cuda))
        else:
            off, data = M.csr_to_dia(rp, ci, v)
            runs.append(native.cg_dia(off, data, b, dtype="fp64", tol=1e-10, algorithm="single_reduction",
                                      device=cuda))
    (x, res), (x2, res2) = runs
    assert it_close(res["iterations"], it), (matrix, fmt, res, it)
    assert np.array_equal(x.cpu().numpy(), x2.cpu().numpy())
    assert true_rel(rp, ci, v, b, x.cpu().numpy()) <= 1e-10 * 1.05


def test_cg_single_reduction_fp32_tracks_oracle(native, cuda, oracle):
    rp, ci, v = oracle.gen_tridiag(5000, 2, np.float32)
    b = np.ones(5000, np.float32)
    xo, _, _, _ = oracle.cg(rp, ci, v, b, max_iter=6, static_iter=True)
    x, res = native.cg_csr(rp, ci, v, b, dtype="fp32", max_iter=6, static_iter=True,
                           algorithm="single_reduction", device=cuda)
    assert res["iterations"] == 6
    assert np.allclose(x.cpu().numpy(), xo, rtol=1e-4, atol=1e-6)
