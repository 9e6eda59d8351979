"""Ensembles of independent hydrogen-like propagations advanced together on one GPU.

Each member is an ordinary ``Problem`` with ``CayleyPropagatorGPU`` or ``PamPropagatorGPU``
(its own basis size, angular size and laser parameters). ``CayleyEnsembleGPU`` binds their
device steppers into a ``pg_cayley_batch``, ``PamEnsembleGPU`` into a ``pg_pamp_batch``: one
CUDA graph launch per ensemble step, one branch per member, the branches running
concurrently (the pAMP exponentials of all members in one kernel between the branches). This is the ensemble mode the reference runs as separate
processes (one job per field parameter set, ``pyprop/utilities/submitpbs*.py``).

``partition_members`` splits an ensemble over ranks for multi-GPU runs (members are
independent: no collective on the data path).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from ._native import check


def partition_members(nmembers, world_size, rank):
    """Contiguous, balanced member ranges: rank r gets [start, stop)."""
    base, extra = divmod(nmembers, world_size)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def gather_member_values(values, nmembers, world_size, rank):
    """Per-member values of this rank's range (partition_members order) gathered into the
    whole ensemble's member order on every rank (torch.distributed; no data-path exchange:
    called once after the timed steps). One rank returns ``values`` unchanged."""
    a, b = partition_members(nmembers, world_size, rank)
    if len(values) != b - a:
        raise ValueError("rank %d holds members [%d, %d) but gave %d values" % (rank, a, b, len(values)))
    if world_size == 1:
        return list(values)
    import torch.distributed as dist
    parts = [None] * world_size
    dist.all_gather_object(parts, list(values))
    out = [v for part in parts for v in part]
    if len(out) != nmembers:
        raise RuntimeError("gathered %d member values, expected %d" % (len(out), nmembers))
    return out


def job_throughput(local_units, local_seconds, world_size):
    """Whole-job units per second of ranks that ran independently: the units summed over the
    ranks divided by the slowest rank's time (torch.distributed SUM and MAX reductions)."""
    if world_size == 1:
        return local_units / local_seconds, local_units, local_seconds
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    units = torch.tensor([float(local_units)], dtype=torch.float64, device=dev)
    secs = torch.tensor([float(local_seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    dist.all_reduce(secs, op=dist.ReduceOp.MAX)
    return units.item() / secs.item(), units.item(), secs.item()


def hydrogen_ensemble_params(nmembers=256, seed=20261203, lmax_range=(8, 32), n_range=(100, 400),
                             e0_range=(0.01, 0.1), wavelength_range=(400.0, 1600.0)):
    """Member parameters drawn from numpy's default_rng(seed): lmax ~ U{8..32}, B-splines
    ~ U{100..400}, peak field ~ U[0.01, 0.1] a.u., wavelength ~ U[400, 1600] nm."""
    rng = np.random.default_rng(seed)
    lmax = rng.integers(lmax_range[0], lmax_range[1] + 1, nmembers)
    nb = rng.integers(n_range[0], n_range[1] + 1, nmembers)
    e0 = rng.uniform(e0_range[0], e0_range[1], nmembers)
    lam = rng.uniform(wavelength_range[0], wavelength_range[1], nmembers)
    return [dict(lmax=int(a), nbsplines=int(b), amplitude=float(c), wavelength_nm=float(d))
            for a, b, c, d in zip(lmax, nb, e0, lam)]


class CayleyEnsembleGPU:
    """Advance many ``Problem`` objects (CayleyPropagatorGPU, same dt) with one launch per step."""

    def __init__(self, problems):
        self.problems = list(problems)
        if not self.problems:
            raise ValueError("empty ensemble")
        props = [p.Propagator for p in self.problems]
        for pr in props:
            if not hasattr(pr, "stepper"):
                raise ValueError("call SetupStep() on every member first")
        self.lib = props[0].stepper.lib
        self.ctx = props[0].stepper.ctx
        n = len(props)
        arr = (C.c_void_p * n)(*[pr.stepper.h.value for pr in props])
        h = C.c_void_p()
        check(self.lib.pg_cayley_batch_create(arr, n, C.byref(h)), "pg_cayley_batch_create")
        self.h = h
        self._keep = props
        self.nslots = props[0].op64.nslots
        if any(pr.op64.nslots != self.nslots for pr in props):
            raise ValueError("ensemble members must have the same number of potential slots")
        self.dt = self.problems[0].TimeStep
        self._psis = (C.c_void_p * n)(*[p.psi.GetData().data_ptr() for p in self.problems])
        self.stats = (nat.KrylovStats * n)()

    def scales(self):
        """(n, nslots) slot values of each member's H(t + dt/2) at its current time."""
        dt = self.dt
        return np.stack([p.Propagator.op64.scales(p.PropagatedTime + abs(dt / 2.0)) for p in self.problems])

    def AdvanceStep(self, scales=None):
        sc = np.ascontiguousarray(self.scales() if scales is None else scales, dtype=np.complex128)
        self.ctx.bind_stream()
        check(self.lib.pg_cayley_batch_step(self.h, self._psis, float(self.dt), sc.view(np.float64).ctypes.data_as(
            nat._DP), self.nslots), "pg_cayley_batch_step")
        for p in self.problems:
            p.PropagatedTime += self.dt

    def scale_table(self, nsteps):
        """Slot values for the next ``nsteps`` steps of every member: (nsteps, n, nslots)."""
        dt = self.dt
        out = np.empty((nsteps, len(self.problems), self.nslots), dtype=np.complex128)
        for k, p in enumerate(self.problems):
            op = p.Propagator.op64
            for s in range(nsteps):
                out[s, k] = op.scales(p.PropagatedTime + s * dt + abs(dt / 2.0))
        return out

    def Stats(self):
        self.ctx.bind_stream()
        check(self.lib.pg_cayley_batch_stats(self.h, self.stats), "pg_cayley_batch_stats")
        return [s.as_dict() for s in self.stats]

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_cayley_batch_destroy(self.h)
        except Exception:
            pass


class PamEnsembleGPU(CayleyEnsembleGPU):
    """Advance many ``Problem`` objects (PamPropagatorGPU, same dt) with one launch per step;
    each member's H is frozen at the step start, as in PamPropagatorGPU.AdvanceStep."""

    def __init__(self, problems):
        self.problems = list(problems)
        if not self.problems:
            raise ValueError("empty ensemble")
        props = [p.Propagator for p in self.problems]
        for pr in props:
            if not hasattr(pr, "stepper"):
                raise ValueError("call SetupStep() on every member first")
        self.lib = props[0].stepper.lib
        self.ctx = props[0].stepper.ctx
        n = len(props)
        arr = (C.c_void_p * n)(*[pr.stepper.h.value for pr in props])
        h = C.c_void_p()
        check(self.lib.pg_pamp_batch_create(arr, n, C.byref(h)), "pg_pamp_batch_create")
        self.h = h
        self._keep = props
        self.nslots = props[0].op64.nslots
        if any(pr.op64.nslots != self.nslots for pr in props):
            raise ValueError("ensemble members must have the same number of potential slots")
        self.dt = self.problems[0].TimeStep
        self._psis = (C.c_void_p * n)(*[p.psi.GetData().data_ptr() for p in self.problems])
        self.stats = (nat.KrylovStats * n)()

    def scales(self):
        """(n, nslots) slot values of each member's H at its current time."""
        return np.stack([p.Propagator.op64.scales(p.PropagatedTime) for p in self.problems])

    def AdvanceStep(self, scales=None):
        sc = np.ascontiguousarray(self.scales() if scales is None else scales, dtype=np.complex128)
        self.ctx.bind_stream()
        check(self.lib.pg_pamp_batch_step(self.h, self._psis, float(self.dt), sc.view(np.float64).ctypes.data_as(
            nat._DP), self.nslots), "pg_pamp_batch_step")
        for p in self.problems:
            p.PropagatedTime += self.dt

    def Stats(self):
        self.ctx.bind_stream()
        check(self.lib.pg_pamp_batch_stats(self.h, self.stats), "pg_pamp_batch_stats")
        return [s.as_dict() for s in self.stats]

    def set_persistent(self, on=True):
        """Force one persistent kernel per ensemble step (True; every member must qualify:
        complex64 basis of at most 20 vectors, rank-2 operator with real bands, band half-width
        at most 8), the graph of every member's kernels (False), or let the first step time both
        and keep the faster (None, the default)."""
        mode = -1 if on is None else (1 if on else 0)
        check(self.lib.pg_pamp_batch_set_mode(self.h, mode), "pg_pamp_batch_set_mode")

    def launch_shape(self):
        """{"persistent", "threads", "ctas", "persistent_ms", "graph_ms"}: the step in use, the
        autotuned launch shape and the timed ensemble steps (zeros before the first step)."""
        mode, th, ct, ms, gms = C.c_int(), C.c_int(), C.c_int(), C.c_float(), C.c_float()
        check(self.lib.pg_pamp_batch_get_mode(self.h, C.byref(mode), C.byref(th), C.byref(ct), C.byref(ms),
                                              C.byref(gms)), "pg_pamp_batch_get_mode")
        return {"persistent": bool(mode.value), "threads": th.value, "ctas": ct.value, "persistent_ms": ms.value,
                "graph_ms": gms.value}

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_pamp_batch_destroy(self.h)
        except Exception:
            pass
