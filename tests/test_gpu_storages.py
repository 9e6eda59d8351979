"""GPU fused operator in every storage of the generated multiply kernels vs the oracle."""
import numpy as np
import pytest

from pyprop_gb300 import _native as nat
from tests.helpers import FakePotential, INNER_KINDS, OUTER_KINDS, random_storage_term, relerr

pytestmark = pytest.mark.gpu

NANG, N, KB = 6, 70, 6


@pytest.mark.parametrize("outer", OUTER_KINDS)
def test_storage_matvec_fp64_fp32(gpu, outer):
    import torch
    from oracle.operators import TermOracle
    from pyprop_gb300.gpu import Context, DeviceOperator
    ctx = Context.get()
    rng = np.random.default_rng(11)
    x = rng.standard_normal((NANG, N)) + 1j * rng.standard_normal((NANG, N))
    y0 = rng.standard_normal((NANG, N)) + 1j * rng.standard_normal((NANG, N))
    for k, inner in enumerate(INNER_KINDS):
        sid, pot, pairs = random_storage_term(outer, inner, NANG, N, KB, seed=100 + k)
        # a second term in another slot, so the slot scales are exercised too
        sid2, pot2, pairs2 = random_storage_term("Diag", "BandNH", NANG, N, KB, seed=200 + k)
        ref = y0.copy()
        TermOracle(sid, pot, pairs, NANG, N, KB).multiply(x, ref, 0.7 - 0.2j)
        TermOracle(sid2, pot2, pairs2, NANG, N, KB).multiply(x, ref, 1.3)
        for prec, dt, tol in [(nat.PG_FP64, torch.complex128, 1e-13), (nat.PG_FP32, torch.complex64, 2e-5)]:
            op = DeviceOperator(ctx, [FakePotential(sid, pot, pairs), FakePotential(sid2, pot2, pairs2)],
                                (NANG, N), KB, prec)
            src = torch.as_tensor(x, device="cuda").to(dt)
            dst = torch.as_tensor(y0, device="cuda").to(dt)
            op.matvec(np.array([0.0, 0.7 - 0.2j, 1.3]), src, dst, accumulate=True)
            got = dst.to(torch.complex128).cpu().numpy()
            assert relerr(got, ref) < tol, (sid, prec, relerr(got, ref))


@pytest.mark.parametrize("storage", ["Diag_Simp_BandNH", "Simp_Simp_BandNH", "Herm_Simp_BandNH", "Diag_Simp_Simp",
                                     "Simp_Diag_Band"])
def test_rank3_matvec_fp64_fp32(gpu, storage):
    import torch
    from oracle.operators import TermOracle
    from pyprop_gb300.gpu import Context, DeviceOperator
    from tests.test_storages import rank3_case
    pot, pairs, shape, kb = rank3_case(storage, nang=4, N=24, kb=3, seed=9)
    # two-electron shape; the angular pair list must stay inside nang = 4
    ctx = Context.get()
    rng = np.random.default_rng(12)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = np.zeros(shape, dtype=np.complex128)
    TermOracle(storage, pot, pairs, None, None, kb, shape=shape).multiply(x, ref, 0.9 + 0.1j)
    for prec, dt, tol in [(nat.PG_FP64, torch.complex128, 1e-13), (nat.PG_FP32, torch.complex64, 2e-5)]:
        op = DeviceOperator(ctx, [FakePotential(storage, pot, pairs)], shape, kb, prec)
        src = torch.as_tensor(x, device="cuda").to(dt)
        dst = torch.zeros(shape, dtype=dt, device="cuda")
        op.matvec(np.array([0.0, 0.9 + 0.1j]), src, dst)
        got = dst.to(torch.complex128).cpu().numpy()
        assert relerr(got, ref) < tol, (storage, prec, relerr(got, ref))


def test_long_fibre_matvec_uses_wide_tiles(gpu):
    """N >= 1024 takes the 128-row bulk-copy tiles (and a partial last tile): parity with the oracle."""
    import torch
    from oracle.operators import TermOracle
    from pyprop_gb300.gpu import Context, DeviceOperator
    nang, N, kb = 5, 1100, 6
    ctx = Context.get()
    terms = [random_storage_term("Diag", "BandNH", nang, N, kb, seed=31),
             random_storage_term("Simp", "BandNH", nang, N, kb, seed=32)]
    rng = np.random.default_rng(33)
    x = rng.standard_normal((nang, N)) + 1j * rng.standard_normal((nang, N))
    ref = np.zeros_like(x)
    for (sid, pot, pairs), s in zip(terms, (1.0, 0.3 - 0.4j)):
        TermOracle(sid, pot, pairs, nang, N, kb).multiply(x, ref, s)
    for prec, dt, tol in [(nat.PG_FP64, torch.complex128, 1e-13), (nat.PG_FP32, torch.complex64, 2e-5)]:
        op = DeviceOperator(ctx, [FakePotential(*t) for t in terms], (nang, N), kb, prec)
        tuned, times = op.variant()
        assert tuned in range(1, 9) and all(t > 0 for t in times[:3])
        # 4, 5, 7, 8 (TMA) when the tensor map exists; 6 builds its row-major band copy on demand
        variants = ((1, 2, 3, 4, 5, 7, 8) if times[3] > 0 else (1, 2, 3)) + (6,)
        src = torch.as_tensor(x, device="cuda").to(dt)
        outs = []
        for v in variants:  # every kernel variant, then back to the tuned one
            op.variant(v)
            dst = torch.zeros((nang, N), dtype=dt, device="cuda")
            op.matvec(np.array([0.0, 1.0, 0.3 - 0.4j]), src, dst)
            outs.append(dst.to(torch.complex128).cpu().numpy())
            assert relerr(outs[-1], ref) < tol, (prec, v)
        assert all(np.array_equal(outs[0], o) for o in outs[1:])
        op.variant(tuned)
