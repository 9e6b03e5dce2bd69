"""MatrixMarket reading (host code of the library, no GPU), checked against
the reference's reading rules: symmetric entries mirrored (negated for
skew-symmetric), pattern values 1.0, rows and columns sorted with duplicates
kept, array files column-major; and against scipy's reader."""
import numpy as np
import pytest


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def dense(rp, ci, v, n, m):
    a = np.zeros((n, m))
    for i in range(n):
        for j in range(rp[i], rp[i + 1]):
            a[i, ci[j]] += v[j]
    return a


def test_general_sorted_with_duplicates(native, tmp_path):
    from perks_gb300.matrices import read_mtx
    p = write(tmp_path, "g.mtx", "%%MatrixMarket matrix coordinate real general\n% comment\n3 4 5\n"
                                 "3 1 2.5\n1 4 -1\n1 2 7\n3 1 0.5\n2 2 4e-3\n")
    rp, ci, v = read_mtx(p)
    assert list(rp) == [0, 2, 3, 5]
    assert list(ci) == [1, 3, 1, 0, 0]
    assert list(v) == [7.0, -1.0, 4e-3, 2.5, 0.5]  # stable: file order among duplicates


def test_symmetric_and_skew_are_mirrored(native, tmp_path):
    from perks_gb300.matrices import read_mtx
    sym = write(tmp_path, "s.mtx", "%%MatrixMarket matrix coordinate real symmetric\n3 3 4\n1 1 4\n2 1 -1\n3 2 -2\n3 3 5\n")
    rp, ci, v = read_mtx(sym)
    a = dense(rp, ci, v, 3, 3)
    assert np.array_equal(a, np.array([[4, -1, 0], [-1, 0, -2], [0, -2, 5.0]]))
    assert rp[-1] == 6
    skew = write(tmp_path, "k.mtx", "%%MatrixMarket matrix coordinate real skew-symmetric\n2 2 1\n2 1 3\n")
    rp, ci, v = read_mtx(skew)
    assert np.array_equal(dense(rp, ci, v, 2, 2), np.array([[0, -3], [3, 0.0]]))


def test_pattern_and_array(native, tmp_path):
    from perks_gb300.matrices import read_mtx
    pat = write(tmp_path, "p.mtx", "%%MatrixMarket matrix coordinate pattern general\n2 3 2\n1 3\n2 1\n")
    rp, ci, v = read_mtx(pat)
    assert list(rp) == [0, 1, 2] and list(ci) == [2, 0] and list(v) == [1.0, 1.0]
    arr = write(tmp_path, "a.mtx", "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    rp, ci, v = read_mtx(arr)
    assert np.array_equal(dense(rp, ci, v, 2, 2), np.array([[1, 3], [2, 4.0]]))


def test_matches_scipy(native, tmp_path):
    sio = pytest.importorskip("scipy.io")
    sp = pytest.importorskip("scipy.sparse")
    from perks_gb300.matrices import random_spd, read_mtx
    rp, ci, v = random_spd(500, 3)
    A = sp.csr_matrix((v, ci, rp), shape=(500, 500))
    p = str(tmp_path / "r.mtx")
    sio.mmwrite(p, A, symmetry="symmetric")
    r2, c2, v2 = read_mtx(p)
    B = sp.csr_matrix((v2, c2, r2), shape=(500, 500))
    assert (abs(A - B) > 1e-12 * abs(A).max()).nnz == 0
    assert all(np.all(np.diff(c2[r2[i]:r2[i + 1]]) > 0) for i in range(500))


def test_errors_are_reported(native, tmp_path):
    from perks_gb300 import PerksError
    from perks_gb300.matrices import read_mtx
    with pytest.raises(PerksError):
        read_mtx(str(tmp_path / "missing.mtx"))
    bad = write(tmp_path, "b.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n")
    with pytest.raises(PerksError):
        read_mtx(bad)


@pytest.mark.gpu
def test_cg_on_a_market_file(native, cuda, oracle, tmp_path):
    """The reference's workflow: a symmetric MatrixMarket file, read, solved by CG."""
    sio = pytest.importorskip("scipy.io")
    sp = pytest.importorskip("scipy.sparse")
    from perks_gb300.matrices import random_spd, read_mtx
    rp, ci, v = random_spd(4000, 9)
    p = str(tmp_path / "spd.mtx")
    sio.mmwrite(p, sp.csr_matrix((v, ci, rp), shape=(4000, 4000)), symmetry="symmetric")
    rp2, ci2, v2 = read_mtx(p)
    b = np.random.default_rng(3).uniform(-1, 1, 4000)
    _, it, _, _ = oracle.cg(rp2, ci2, v2, b, max_iter=20000, stop=1, tol=1e-10)
    x, res = native.cg_csr(rp2, ci2, v2, b, dtype="fp64", tol=1e-10, device=cuda)
    assert abs(res["iterations"] - it) <= max(1, int(0.01 * it))
    assert res["true_rel_res"] <= 1.05e-10
