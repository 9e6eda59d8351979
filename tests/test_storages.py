"""Storage layouts of the generated multiply kernels, checked on the oracle (CPU).

Each angular storage (Simp, Herm, Diag, Ident, Band, BandNH, Dense) and radial storage
(BandNH, Band, Dense, Diag, Ident) of core/tensorpotential/tensorpotentialmultiply_generator.py
is pinned against another one holding the same matrix, so a wrong index map in any of
them shows up as a mismatch.
"""
import numpy as np
import pytest

from oracle.operators import TermOracle, dense_operator, outer_blocks
from tests.helpers import random_storage_term

NANG, N, KB = 5, 40, 3


def dense_of(storage, pot, pairs):
    return dense_operator([TermOracle(storage, pot, pairs, NANG, N, KB)], [1.0], NANG, N)


def bandnh_index_loop(n, bc):
    """The three BandNH loops of the generator (:662-694) stepped literally: (row, col) -> i."""
    sub = (bc - 1) // 2
    idx = {}
    i = 0
    for col in range(0, sub):
        i += sub - col
        for row in range(0, col + sub + 1):
            idx[(row, col)] = i
            i += 1
    for col in range(sub, n - sub):
        for row in range(col - sub, col + sub + 1):
            idx[(row, col)] = i
            i += 1
    for col in range(n - sub, n):
        for row in range(col - sub, n):
            idx[(row, col)] = i
            i += 1
        i += -n + col + sub + 1
    return idx


@pytest.mark.parametrize("n,bc", [(7, 3), (9, 5), (6, 1)])
def test_bandnh_outer_index_map_matches_generator_loops(n, bc):
    blocks = outer_blocks("BandNH", n * bc, None, n)
    assert {(r, c): i for r, c, i, _ in blocks} == bandnh_index_loop(n, bc)


def test_herm_equals_simp_with_mirrored_conjugated_pairs():
    for inner in ("BandNH", "Dense", "Diag", "Ident"):
        sid, pot, pairs = random_storage_term("Herm", inner, NANG, N, KB, seed=1)
        M = dense_of(sid, pot, pairs)
        pairs2 = np.concatenate([pairs, pairs[:, ::-1]])
        M2 = dense_of("Simp_" + inner, np.concatenate([pot, pot.conj()]), pairs2)
        assert np.abs(M - M2).max() < 1e-14, inner


def test_dense_outer_equals_simp_over_all_pairs():
    sid, pot, _ = random_storage_term("Dense", "BandNH", NANG, N, KB, seed=2)
    pairs = np.array([(r, c) for r in range(NANG) for c in range(NANG)], dtype=np.int32)
    assert np.abs(dense_of(sid, pot, None) - dense_of("Simp_BandNH", pot, pairs)).max() < 1e-14


def test_band_outer_is_hermitian_for_hermitian_blocks():
    # Band angular storage holds the upper blocks; the mirrored lower blocks are their
    # conjugates, so real symmetric radial blocks give a Hermitian operator
    sid, pot, _ = random_storage_term("Band", "Diag", NANG, N, KB, seed=3, outer_band=3)
    bc = pot.shape[0] // NANG
    pot[::bc] = pot[::bc].real  # angular diagonal blocks Hermitian (real diagonal)
    M = dense_of(sid, pot, None)
    assert np.abs(M - M.conj().T).max() < 1e-14
    # element (row, col >= row) of the angular band comes from slot row*bc + (col-row)
    r, c = 1, 3
    assert np.allclose(np.diag(M[r * N:(r + 1) * N, c * N:(c + 1) * N]), pot[r * bc + (c - r)])


def test_radial_storages_agree_on_one_hermitian_band_matrix():
    rng = np.random.default_rng(4)
    A = np.zeros((N, N), dtype=np.complex128)
    for d in range(0, KB + 1):
        v = rng.standard_normal(N - d) + 1j * rng.standard_normal(N - d)
        A[np.arange(d, N), np.arange(N - d)] = v  # lower diagonal d
    A = A + A.conj().T
    # BandNH: slot j*(2kb+1) + kb + i - j
    b = 2 * KB + 1
    bandnh = np.zeros(N * b, dtype=np.complex128)
    band = np.zeros(N * (KB + 1), dtype=np.complex128)
    for i in range(N):
        for j in range(max(0, i - KB), min(N, i + KB + 1)):
            bandnh[j * b + KB + i - j] = A[i, j]
            if i >= j:
                band[j * (KB + 1) + i - j] = A[i, j]
    dense = A.reshape(1, -1)
    Ms = [dense_of("Diag_BandNH", np.repeat(bandnh[None], NANG, 0), None),
          dense_of("Diag_Band", np.repeat(band[None], NANG, 0), None),
          dense_of("Diag_Dense", np.repeat(dense, NANG, 0), None)]
    for M in Ms[1:]:
        assert np.abs(M - Ms[0]).max() < 1e-13
    assert np.abs(Ms[0][:N, :N] - A).max() < 1e-14


def test_band_radial_ignores_imaginary_diagonal_and_conjugate_flag():
    # zhbmv reads only the real part of the diagonal and the reference calls it for the
    # mirrored Herm half as well (no conjugation)
    sid, pot, pairs = random_storage_term("Herm", "Band", NANG, N, KB, seed=5)
    t = TermOracle(sid, pot, pairs, NANG, N, KB)
    half = len(pairs)
    assert np.abs(t.bands[:half] - t.bands[half:]).max() == 0.0
    assert np.all(t.bands[:, :, KB].imag == 0.0)


@pytest.mark.parametrize("outer", ["Simp", "Herm", "Diag", "Ident", "Band", "BandNH", "Dense"])
def test_multiply_matches_dense_assembly(outer):
    for inner in ("BandNH", "Band", "Dense", "Diag", "Ident"):
        sid, pot, pairs = random_storage_term(outer, inner, NANG, N, KB, seed=6)
        t = TermOracle(sid, pot, pairs, NANG, N, KB)
        x = np.random.default_rng(7).standard_normal((NANG, N)) + 0j
        y = np.zeros_like(x)
        t.multiply(x, y, 0.5)
        M = dense_operator([t], [0.5], NANG, N)
        assert np.abs(y.ravel() - M @ x.ravel()).max() < 1e-12, sid


# ---------------------------------------------------------------------------------------
# rank 3: [Nang][N][N] two-electron layout
# ---------------------------------------------------------------------------------------
def packed_pairs(n, k):
    """banded-packed pairs (basis/BSpline.py:25-44): row-major, |i-j| < k."""
    return np.array([(i, j) for i in range(n) for j in range(max(0, i - k + 1), min(n, i + k))], dtype=np.int32)


def rank3_case(storage, nang=3, N=9, kb=2, seed=0):
    rng = np.random.default_rng(seed)
    k0, k1, k2 = storage.split("_")
    ang_pairs = np.array([(0, 0), (0, 1), (1, 0), (1, 2), (2, 2)], dtype=np.int32)
    r1_pairs = packed_pairs(N, kb + 1)
    r2_pairs = packed_pairs(N, kb + 1)
    e0 = {"Diag": nang, "Simp": len(ang_pairs), "Herm": len(ang_pairs)}[k0]
    e1 = {"Simp": len(r1_pairs), "Diag": N}[k1]
    e2 = {"BandNH": N * (2 * kb + 1), "Band": N * (kb + 1), "Simp": len(r2_pairs)}[k2]
    pot = rng.standard_normal((e0, e1, e2)) + 1j * rng.standard_normal((e0, e1, e2))
    pairs = [ang_pairs if k0 in ("Simp", "Herm") else None, r1_pairs if k1 == "Simp" else None,
             r2_pairs if k2 == "Simp" else None]
    return pot, pairs, (nang, N, N), kb


def direct_rank3(storage, pot, pairs, shape, kb):
    """Dense operator from the generated loops written out as three nested loops."""
    nang, N, _ = shape
    k0, k1, k2 = storage.split("_")
    M = np.zeros((nang * N * N, nang * N * N), dtype=np.complex128)

    def rank_loop(kind, pr, n):
        if kind == "Diag":
            return [(a, a, a, False) for a in range(n)]
        out = [(int(r), int(c), p, False) for p, (r, c) in enumerate(pr)]
        if kind == "Herm":
            out += [(int(c), int(r), p, True) for p, (r, c) in enumerate(pr)]
        return out

    for a_r, a_c, ia, c0 in rank_loop(k0, pairs[0], nang):
        for i_r, i_c, i1, c1 in rank_loop(k1, pairs[1], N):
            v = pot[ia, i1]
            conj = c0 != c1
            blk = np.zeros((N, N), dtype=np.complex128)
            if k2 == "BandNH":
                b = 2 * kb + 1
                for i in range(N):
                    for j in range(max(0, i - kb), min(N, i + kb + 1)):
                        blk[i, j] = v[j * b + kb + i - j]
                if conj:
                    blk = blk.conj()
            elif k2 == "Band":  # zhbmv('L'), conjugate flag ignored, diagonal real
                for i in range(N):
                    for j in range(max(0, i - kb), i + 1):
                        blk[i, j] = v[j * (kb + 1) + i - j]
                        blk[j, i] = np.conj(blk[i, j])
                    blk[i, i] = blk[i, i].real
            else:  # Simp
                for p, (i, j) in enumerate(pairs[2]):
                    blk[i, j] += np.conj(v[p]) if conj else v[p]
            r0 = (a_r * N + i_r) * N
            c0_ = (a_c * N + i_c) * N
            M[r0:r0 + N, c0_:c0_ + N] += blk
    return M


@pytest.mark.parametrize("storage", ["Diag_Simp_BandNH", "Simp_Simp_BandNH", "Herm_Simp_BandNH", "Diag_Simp_Simp",
                                     "Simp_Diag_Band", "Herm_Simp_Simp"])
def test_rank3_oracle_matches_direct_loops(storage):
    pot, pairs, shape, kb = rank3_case(storage)
    t = TermOracle(storage, pot, pairs, None, None, kb, shape=shape)
    M = dense_operator([t], [1.0], shape[0] * shape[1], shape[2])
    assert np.abs(M - direct_rank3(storage, pot, pairs, shape, kb)).max() < 1e-13
    x = np.random.default_rng(3).standard_normal(shape) + 0j
    y = np.zeros(shape, dtype=np.complex128)
    t.multiply(x, y, 2.0)
    assert np.abs(y.ravel() - 2.0 * M @ x.ravel()).max() < 1e-12


def test_empty_pair_list_term():
    # lmax = 0: the dipole term has no angular pairs and adds nothing
    pot = np.zeros((0, N * (2 * KB + 1)), dtype=np.complex128)
    t = TermOracle("Simp_BandNH", pot, np.zeros((0, 2), dtype=np.int32), 1, N, KB)
    y = np.zeros((1, N), dtype=np.complex128)
    t.multiply(np.ones((1, N), dtype=np.complex128), y, 1.0)
    assert not y.any() and len(t.rows) == 0
