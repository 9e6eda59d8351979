"""Python handles over the C ABI: context, fused operator, banded fibre operators and the
Krylov steppers. Device buffers are torch tensors on the current CUDA device; the library
runs on torch's current stream so its kernels are ordered with torch's.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from ._native import check

_TORCH = None


def torch():
    global _TORCH
    if _TORCH is None:
        import torch as _t
        _TORCH = _t
    return _TORCH


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise RuntimeError("pyprop_gb300 needs a CUDA device: the GPU path has no CPU fallback")


def ptr(tensor):
    return C.c_void_p(tensor.data_ptr())


class Context:
    """One pg_ctx per CUDA device, bound to torch's current stream at each use."""

    _instances: dict = {}

    def __init__(self, device=0):
        require_cuda()
        self.lib = nat.load()
        h = C.c_void_p()
        check(self.lib.pg_ctx_create(device, C.byref(h)), "pg_ctx_create")
        self.h = h
        self.device = device

    @classmethod
    def get(cls, device=None):
        t = torch()
        if device is None:
            device = t.cuda.current_device()
        if device not in cls._instances:
            cls._instances[device] = Context(device)
        ctx = cls._instances[device]
        ctx.bind_stream()
        return ctx

    def bind_stream(self):
        """Bind the context to torch's current stream on its device (called before every
        launch; the raw-handle query avoids building a Stream object each time)."""
        t = torch()
        raw = getattr(t._C, "_cuda_getCurrentRawStream", None)
        s = raw(self.device) if raw is not None else t.cuda.current_stream(self.device).cuda_stream
        check(self.lib.pg_ctx_set_stream(self.h, C.c_void_p(s)), "pg_ctx_set_stream")

    def launches(self):
        return int(self.lib.pg_ctx_kernel_launches(self.h))

    def synchronize(self):
        check(self.lib.pg_ctx_synchronize(self.h), "pg_ctx_synchronize")

    def device_error(self):
        """The device error flag (0: clear; set by a bounded wait that ran out). Waits."""
        flag = C.c_int(0)
        self.bind_stream()
        check(self.lib.pg_ctx_device_error(self.h, C.byref(flag)), "pg_ctx_device_error")
        return int(flag.value)

    def clear_device_error(self):
        self.bind_stream()
        check(self.lib.pg_ctx_clear_device_error(self.h), "pg_ctx_clear_device_error")


def complex_dtype(precision):
    t = torch()
    return t.complex128 if precision == nat.PG_FP64 else t.complex64


def precision_of(name):
    name = (name or "fp64").lower()
    if name in ("fp64", "double", "complex128"):
        return nat.PG_FP64
    if name in ("fp32", "single", "complex64", "mixed"):
        return nat.PG_FP32
    raise ValueError("unknown precision %r" % (name,))


def bandnh_from_rows(rows, kb):
    """(N, 2kb+1) row-oriented band -> reference BandNH layout (N*(2kb+1),), complex128."""
    N = rows.shape[0]
    b = 2 * kb + 1
    out = np.zeros(N * b, dtype=np.complex128)
    for d in range(-kb, kb + 1):
        i = np.arange(max(0, -d), min(N, N - d))
        j = i + d
        out[j * b + (kb + i - j)] = rows[i, kb + d]
    return out


class DeviceOperator:
    """Fused sum of tensor potentials (and optionally S) resident on the device.

    Slots: 0 is the overlap S when ``overlap_rows`` is given; potential ``p`` uses slot
    ``1 + p``. ``scales(t)`` gives the slot values of H(t) (time functions evaluated on
    the host, as the reference does per matvec).
    """

    def __init__(self, ctx, potentials, shape, kb, precision, overlap_rows=None, fp64_emulation=False):
        self.ctx = ctx
        self.lib = ctx.lib
        self.shape = tuple(shape)
        self.kb = kb
        self.precision = precision
        self.potentials = list(potentials)
        if 1 + len(self.potentials) > 16:
            raise ValueError("at most 15 consolidated potentials per operator")
        h = C.c_void_p()
        shp, shp_p = nat.iptr(np.asarray(shape, dtype=np.int32))
        check(self.lib.pg_op_create(ctx.h, len(shape), shp_p, kb, precision, C.byref(h)), "pg_op_create")
        self.h = h
        self.fp64_emulation = bool(fp64_emulation) and precision == nat.PG_FP64
        if self.fp64_emulation:
            check(self.lib.pg_op_set_fp64_emulation(self.h, 1), "pg_op_set_fp64_emulation")
        self.has_overlap = overlap_rows is not None
        any_factored = any(getattr(pot, "Factors", None) is not None for pot in self.potentials)
        overlap_factor = None
        if overlap_rows is not None:
            rows = np.asarray(overlap_rows, dtype=np.float64)
            band = bandnh_from_rows(rows, kb)[None, :]
            if len(shape) == 3 and any_factored:
                # two electrons with factorized terms: S x S as one more factor (identity on the
                # channels, S[i1][d1] S[i2][d2] on the radial grid)
                overlap_factor = np.einsum("ad,ce->adec", rows, rows)
            elif len(shape) == 2:
                self._add(["Ident", "BandNH"], band, [None, None], 0)
            else:
                # two electrons: S x S on the radial ranks, the first one as a packed pair list
                N = rows.shape[0]
                pr = np.array([(i, j) for i in range(N) for j in range(max(0, i - kb), min(N, i + kb + 1))],
                              dtype=np.int32)
                s1 = rows[pr[:, 0], kb + pr[:, 1] - pr[:, 0]]
                self._add(["Ident", "Simp", "BandNH"], (s1[:, None] * band)[None], [None, pr, None], 0)
        factored = []
        for p, pot in enumerate(self.potentials):
            if getattr(pot, "Factors", None) is not None:
                factored.append((pot.Factors, 1 + p))
                continue
            kinds = [g.GetStorageId() for g in pot.GeometryList]
            pairs = [g.GetBasisPairs() if k in ("Simp", "Herm") else None for g, k in zip(pot.GeometryList, kinds)]
            self._add(kinds, pot.PotentialData, pairs, 1 + p)
        self.nfactors = 0
        if overlap_factor is not None:
            from .tensorpotential import FactoredPotential
            factored.insert(0, (FactoredPotential(None, np.ones((1, shape[0])), np.ones(1, dtype=np.complex128),
                                                  overlap_factor[None], None, kb, shape[0]), 0))
        if factored:
            self._add_factored(factored)
        check(self.lib.pg_op_finalize(self.h), "pg_op_finalize")

    def _add_factored(self, factored):
        """All factors of the factorized terms in one call; factors with the same slot, weight
        and angular coefficients (the radial kinetic energies and the nuclear attraction, all
        1 on the diagonal) are summed into one radial operator."""
        merged = {}
        order = []
        for fac, slot in factored:
            rows, cols = fac.entries()
            for q in range(fac.nfactors):
                c = fac.coefs[q]
                nz = np.nonzero(c)[0]
                key = (slot, complex(fac.weights[q]), rows[nz].tobytes(), cols[nz].tobytes(), c[nz].tobytes())
                if key in merged:
                    merged[key][0] = merged[key][0] + fac.stencil[q]
                else:
                    merged[key] = [fac.stencil[q], rows[nz], cols[nz], c[nz], slot, complex(fac.weights[q])]
                    order.append(key)
        Q = len(order)
        radial = np.ascontiguousarray(np.stack([merged[k][0] for k in order]), dtype=np.float64)
        weights = np.ascontiguousarray(np.array([merged[k][5] for k in order], dtype=np.complex128))
        slots = np.asarray([merged[k][4] for k in order], dtype=np.int32)
        ef = np.concatenate([np.full(len(merged[k][1]), q, dtype=np.int32) for q, k in enumerate(order)])
        er = np.ascontiguousarray(np.concatenate([merged[k][1] for k in order]), dtype=np.int32)
        ec = np.ascontiguousarray(np.concatenate([merged[k][2] for k in order]), dtype=np.int32)
        ev = np.ascontiguousarray(np.concatenate([merged[k][3] for k in order]), dtype=np.float64)
        _, rp = nat.dptr(radial.reshape(-1))
        _, wp = nat.dptr(weights.view(np.float64))
        _, sp = nat.iptr(slots)
        _, fp = nat.iptr(ef)
        _, rowp = nat.iptr(er)
        _, colp = nat.iptr(ec)
        _, vp = nat.dptr(ev)
        check(self.lib.pg_op_add_factored(self.h, Q, rp, wp, sp, len(ev), fp, rowp, colp, vp), "pg_op_add_factored")
        self.nfactors = Q

    def factored_info(self):
        """dict: factors, angular entries, flops of the angular mix and of the radial stencil
        per matvec, bytes of the radial factors and of the per-factor scratch."""
        info = np.zeros(6)
        _, ip = nat.dptr(info)
        check(self.lib.pg_op_factored_info(self.h, ip), "pg_op_factored_info")
        keys = ("factors", "entries", "flops_mix", "flops_radial", "radial_bytes", "scratch_bytes")
        return dict(zip(keys, info.tolist()))

    def _add(self, kinds, data, pairs, slot):
        ids = "_".join(kinds)
        rank = len(kinds)
        data = np.ascontiguousarray(data, dtype=np.complex128)
        if data.ndim != rank:
            data = data.reshape(data.shape[:rank - 1] + (-1,)) if data.ndim > rank else data.reshape((1,) * (rank - data.ndim) + data.shape)
        _, dp = nat.dptr(data.view(np.float64))
        ext = np.asarray(data.shape, dtype=np.int32)
        lists = [np.asarray(pr, dtype=np.int32).reshape(-1, 2) for pr in pairs if pr is not None]
        allp = np.ascontiguousarray(np.concatenate(lists) if lists else np.zeros((0, 2), dtype=np.int32))
        npairs = np.asarray([0 if pr is None else len(np.asarray(pr).reshape(-1, 2)) for pr in pairs], dtype=np.int32)
        _, ep = nat.iptr(ext)
        _, pp = nat.iptr(allp)
        _, npp = nat.iptr(npairs)
        check(self.lib.pg_op_add_term_ranks(self.h, ids.encode(), dp, ep, pp, npp, slot), "pg_op_add_term(%s)" % ids)

    @property
    def nslots(self):
        return 1 + len(self.potentials)

    def scales(self, t, h_factor=1.0, s_weight=0.0):
        sc = np.zeros(self.nslots, dtype=np.complex128)
        sc[0] = s_weight
        for p, pot in enumerate(self.potentials):
            sc[1 + p] = h_factor * pot.GetTimeScaling(t)
        return sc

    def stored_elements(self):
        return int(self.lib.pg_op_stored_elements(self.h))

    def variant(self, force=-1):
        """(variant in use, tuning times in us per variant 1..8; 0 = not offered); force selects one."""
        cur = C.c_int(0)
        times = (C.c_float * 9)()
        check(self.lib.pg_op_variant(self.h, int(force), C.byref(cur), times), "pg_op_variant")
        return cur.value, [float(times[k]) for k in range(1, 9)]

    def matvec(self, scales, src, dst, accumulate=False):
        sc = np.ascontiguousarray(scales, dtype=np.complex128)
        _, sp = nat.dptr(sc.view(np.float64))
        self.ctx.bind_stream()
        check(self.lib.pg_op_matvec(self.h, sp, len(sc), ptr(src), ptr(dst), int(accumulate)), "pg_op_matvec")

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_op_destroy(self.h)
        except Exception:
            pass


class Banded:
    """Overlap factor or block-diagonal preconditioner on the device (pg_banded)."""

    def __init__(self, op: DeviceOperator, h):
        self.op = op
        self.h = h
        self.lib = op.lib

    @classmethod
    def overlap(cls, op, overlap_rows):
        rows, rp = nat.dptr(np.asarray(overlap_rows, dtype=np.float64))
        h = C.c_void_p()
        check(op.lib.pg_overlap_create(op.h, rp, C.byref(h)), "pg_overlap_create")
        return cls(op, h)

    @classmethod
    def blockdiag(cls, op, overlap_rows, cS, cH, slots, weights):
        rows, rp = nat.dptr(np.asarray(overlap_rows, dtype=np.float64))
        cs, csp = nat.dptr(np.array([cS], dtype=np.complex128).view(np.float64))
        ch, chp = nat.dptr(np.array([cH], dtype=np.complex128).view(np.float64))
        sl, slp = nat.iptr(np.asarray(slots, dtype=np.int32))
        wt, wtp = nat.dptr(np.asarray(weights, dtype=np.complex128).view(np.float64))
        h = C.c_void_p()
        check(op.lib.pg_prec_blockdiag_create(op.h, rp, csp, chp, slp, wtp, len(sl), C.byref(h)),
              "pg_prec_blockdiag_create")
        return cls(op, h)

    @classmethod
    def kron(cls, op, overlap_rows, cS, cH, h1, h2):
        """Two-electron Kronecker-factorized radial preconditioner (pg_prec_kron_create)."""
        rows, rp = nat.dptr(np.asarray(overlap_rows, dtype=np.float64))
        cs, csp = nat.dptr(np.array([cS], dtype=np.complex128).view(np.float64))
        ch, chp = nat.dptr(np.array([cH], dtype=np.complex128).view(np.float64))
        a1, a1p = nat.dptr(np.ascontiguousarray(h1, dtype=np.complex128).view(np.float64))
        a2, a2p = nat.dptr(np.ascontiguousarray(h2, dtype=np.complex128).view(np.float64))
        h = C.c_void_p()
        check(op.lib.pg_prec_kron_create(op.h, rp, csp, chp, a1p, a2p, C.byref(h)), "pg_prec_kron_create")
        return cls(op, h)

    @classmethod
    def fast_diagonalization(cls, op, V, lam, lidx, cS, cH):
        """Two-electron radial preconditioner by fast diagonalization (pg_prec_fd_create):
        V [nl][N][N] generalized eigenvectors (columns), lam [nl][N], lidx [Nang][2]."""
        v, vp = nat.dptr(np.ascontiguousarray(V, dtype=np.float64))
        l, lp = nat.dptr(np.ascontiguousarray(lam, dtype=np.float64))
        li, lip = nat.iptr(np.ascontiguousarray(lidx, dtype=np.int32))
        cs, csp = nat.dptr(np.array([cS], dtype=np.complex128).view(np.float64))
        ch, chp = nat.dptr(np.array([cH], dtype=np.complex128).view(np.float64))
        h = C.c_void_p()
        check(op.lib.pg_prec_fd_create(op.h, len(V), vp, lp, lip, csp, chp, C.byref(h)), "pg_prec_fd_create")
        return cls(op, h)

    @staticmethod
    def fast_diagonalization_max_n(ctx, precision):
        return int(ctx.lib.pg_prec_fd_max_n(precision))

    def apply(self, which, x):
        self.op.ctx.bind_stream()
        check(self.lib.pg_banded_apply(self.h, which, ptr(x)), "pg_banded_apply")

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_banded_destroy(self.h)
        except Exception:
            pass


class PampStepper:
    """pg_pamp: one pAMP step per call on a complex128 device wavefunction."""

    def __init__(self, op64, opb, ovl64, ovlb, basis_size, precision, double_ortho=True):
        self.lib = op64.lib
        self.ctx = op64.ctx
        self.op64 = op64
        self._keep = (op64, opb, ovl64, ovlb)
        h = C.c_void_p()
        check(self.lib.pg_pamp_create(op64.h, opb.h, ovl64.h, ovlb.h, basis_size, precision, int(double_ortho),
                                      C.byref(h)), "pg_pamp_create")
        self.h = h
        self.stats = nat.KrylovStats()

    def step(self, psi, dt, scales, want_stats=True):
        """One step; with ``want_stats`` the call waits for it and returns the statistics,
        otherwise it only enqueues (where the exponential runs on the device) and returns None."""
        sc = np.ascontiguousarray(scales, dtype=np.complex128)  # kept alive across the call
        self.ctx.bind_stream()
        check(self.lib.pg_pamp_step(self.h, ptr(psi), float(dt), sc.ctypes.data_as(nat._DP), len(sc),
                                    C.byref(self.stats) if want_stats else None), "pg_pamp_step")
        return self.stats if want_stats else None

    def last_stats(self):
        self.ctx.bind_stream()
        check(self.lib.pg_pamp_last_stats(self.h, C.byref(self.stats)), "pg_pamp_last_stats")
        return self.stats

    def set_fused(self, on):
        """Single-kernel step (complex64 basis; the default where the operators qualify) or the
        graphs. Returns whether the single-kernel step is now selected."""
        code = self.lib.pg_pamp_set_fused(self.h, int(bool(on)))
        if on and code in (nat.PG_ERR_STATE, nat.PG_ERR_STORAGE, nat.PG_ERR_SHAPE):
            return False
        check(code, "pg_pamp_set_fused")
        return bool(on)

    def set_barrier_probe(self, extra_arrivals, at_barrier=0):
        """Test hook: grid barrier number ``at_barrier`` of later single-kernel steps waits for
        arrivals that never come (its bounded polls run out; error word 2)."""
        check(self.lib.pg_pamp_set_barrier_probe(self.h, int(extra_arrivals), int(at_barrier)),
              "pg_pamp_set_barrier_probe")

    def set_device_exp(self, on):
        """Graph path: True runs the m x m exponential on the device (basis of at most 48
        vectors; a step never waits for the host), False (default) on the host between two
        graphs (faster on this GPU, whose FP64 arithmetic is scarce)."""
        check(self.lib.pg_pamp_set_device_exp(self.h, int(bool(on))), "pg_pamp_set_device_exp")

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_pamp_destroy(self.h)
        except Exception:
            pass


class CayleyStepper:
    """pg_cayley: one Crank-Nicolson step per call (GMRES + block-diagonal preconditioner),
    executed as one CUDA graph launch."""

    def __init__(self, op64, opb, prec64, precb, basis_size, precision, tolerance, true_residual=False):
        self.lib = op64.lib
        self.ctx = op64.ctx
        self._keep = (op64, opb, prec64, precb)
        h = C.c_void_p()
        check(self.lib.pg_cayley_create(op64.h, opb.h, prec64.h, precb.h, basis_size, precision, float(tolerance),
                                        C.byref(h)), "pg_cayley_create")
        self.h = h
        check(self.lib.pg_cayley_set_true_residual(h, int(bool(true_residual))), "pg_cayley_set_true_residual")
        self.stats = nat.KrylovStats()

    def step(self, psi, dt, scales, want_stats=True):
        sc = np.ascontiguousarray(scales, dtype=np.complex128)  # kept alive across the call
        self.ctx.bind_stream()
        check(self.lib.pg_cayley_step(self.h, ptr(psi), float(dt), sc.ctypes.data_as(nat._DP), len(sc),
                                      C.byref(self.stats) if want_stats else None), "pg_cayley_step")
        return self.stats if want_stats else None

    def last_stats(self):
        self.ctx.bind_stream()
        check(self.lib.pg_cayley_last_stats(self.h, C.byref(self.stats)), "pg_cayley_last_stats")
        return self.stats

    def set_fused_variant(self, variant):
        """Layout of the single-kernel step: 0 the cluster layout where it fits (default), 1 one
        CTA per channel, 2 the cluster layout (raises where it does not fit)."""
        check(self.lib.pg_cayley_set_fused_variant(self.h, int(variant)), "pg_cayley_set_fused_variant")

    def fused_variant(self):
        """1 or 2: the layout of the next single-kernel step; 0 for the multi-kernel step."""
        v = C.c_int()
        check(self.lib.pg_cayley_get_fused_variant(self.h, C.byref(v)), "pg_cayley_get_fused_variant")
        return v.value

    def totals(self):
        """(GMRES iterations, refinement passes) summed over every step so far (waits)."""
        it, ps = C.c_longlong(), C.c_longlong()
        self.ctx.bind_stream()
        check(self.lib.pg_cayley_totals(self.h, C.byref(it), C.byref(ps)), "pg_cayley_totals")
        return it.value, ps.value

    def set_learned(self, net, coupling_slot):
        """Use the learned preconditioner ``net`` (MlpNet, or None to switch it off); its
        correction is scaled by i dt/2 times the scale of ``coupling_slot``."""
        self.learned_net = net  # keeps the network alive while the stepper uses it
        check(self.lib.pg_cayley_set_learned(self.h, net.h if net is not None else None, int(coupling_slot)),
              "pg_cayley_set_learned")

    def learned_rejected(self):
        out = C.c_longlong(0)
        check(self.lib.pg_cayley_learned_rejected(self.h, C.byref(out)), "pg_cayley_learned_rejected")
        return int(out.value)

    def set_eager(self, on):
        """Host-driven loops instead of the graph's conditional nodes (for profilers)."""
        check(self.lib.pg_cayley_set_eager(self.h, int(bool(on))), "pg_cayley_set_eager")

    def set_fused(self, on):
        """Single-kernel mixed step (the default where the operators qualify) or the captured
        multi-kernel step. Returns whether the single-kernel step is now selected."""
        code = self.lib.pg_cayley_set_fused(self.h, int(bool(on)))
        self.fused_status = code
        if on and code in (nat.PG_ERR_STATE, nat.PG_ERR_STORAGE, nat.PG_ERR_SHAPE):
            return False
        check(code, "pg_cayley_set_fused")
        return bool(on)

    def set_barrier_probe(self, extra_arrivals, at_barrier=0):
        """Test hook: grid barrier number ``at_barrier`` (0 = the first) of later single-kernel
        steps waits for arrivals that never come (its bounded polls run out; error word 2);
        extra_arrivals = 0 restores normal steps."""
        check(self.lib.pg_cayley_set_barrier_probe(self.h, int(extra_arrivals), int(at_barrier)),
              "pg_cayley_set_barrier_probe")

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_cayley_destroy(self.h)
        except Exception:
            pass


def swap_last2(ctx, x, y):
    """y[a][j][i] = x[a][i][j] for rank-3 device tensors (complex128 or complex64)."""
    t = torch()
    prec = nat.PG_FP64 if x.dtype == t.complex128 else nat.PG_FP32
    n0, n1, n2 = x.shape
    ctx.bind_stream()
    check(ctx.lib.pg_vec_swap_last2(ctx.h, prec, ptr(x), ptr(y), n0, n1, n2), "pg_vec_swap_last2")


def vec_dot(ctx, x, y, precision=nat.PG_FP64):
    out = np.zeros(2)
    _, op = nat.dptr(out)
    ctx.bind_stream()
    check(ctx.lib.pg_vec_dot(ctx.h, precision, ptr(x), ptr(y), x.numel(), op), "pg_vec_dot")
    return complex(out[0], out[1])
