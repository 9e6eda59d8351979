"""Benchmark: Cayley/Crank-Nicolson propagation steps per second on one GB300.

Workload (one step = one Crank-Nicolson step of the whole wavefunction): hydrogen,
lmax 40 (41 channels), 600 B-splines of order 7 on an exponential-linear grid r in
[0, 400], Coulomb + length-gauge dipole of an 800 nm sin^2 pulse (peak 0.05 a.u.,
50 a.u. long), dt = 0.01, GMRES (basis 20) left-preconditioned by the block-diagonal
banded LU. The measured path is the mixed-precision one: the residual in FP64, the operator,
Krylov basis, Givens rotations and back-substitution in complex64/FP32, the Gram-Schmidt
and norm sums in FP64, the correction added and the true residual checked in FP64 - one
cooperative kernel per step. Both paths run at equal final-state error: the GMRES tolerance
of each is the loosest that keeps the state after the whole pulse within an infidelity of
1e-8 of the complex128 reference run (mixed 1e-7, plain FP64 1e-6; tests/golden/
run_cayley_l40.npz holds the reference run's final state). Beside the timed steps the whole
5000-step pulse is run on both paths and its infidelity against the reference reported. The
default 5000 steps are the workload's own length (about a second of timed steps, so that the
clock sampler sees the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Rank 0 prints one JSON line. ``--impl reference`` times the CPU oracle port of the
reference algorithm (numpy/scipy complex128, one process per host core, bounded sample).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Cayley propagation steps/s (hydrogen lmax40 N600, mixed FP32/FP64, vs plain FP64 GPU path at equal error)"
WORKLOAD = dict(lmax=40, nbsplines=600, rmax=400.0, timestep=0.01, pulse_duration=50.0, amplitude=0.05,
                wavelength_nm=800.0, krylov_basis_size=20, gmres_tolerance=1e-12)
REFERENCE_RUN = os.path.join(ROOT, "tests", "golden", "run_cayley_l40.npz")


def _config(precision, tolerance=None):
    """The workload's config text; tolerance None = the equal-error GMRES tolerance of the path."""
    from pyprop_gb300.workloads import EQUAL_ERROR_TOLERANCE, hydrogen
    kw = dict(WORKLOAD)
    kw["gmres_tolerance"] = EQUAL_ERROR_TOLERANCE[precision] if tolerance is None else tolerance
    return hydrogen(propagator="CayleyPropagatorGPU", precision=precision, duration=50.0, **kw)


def initial_state(prob):
    """Field-free 1s state of the l = 0 channel (host generalized eigenproblem, setup only)."""
    import scipy.linalg as sl
    repr_ = prob.psi.GetRepresentation()
    nang, N = repr_.GetFullShape()
    bp = prob.Propagator.BasePropagator
    h0 = bp.PotentialList[0].PotentialData[0]
    kb = repr_.kb
    b = 2 * kb + 1
    H = np.zeros((N, N), dtype=complex)
    S = np.zeros((N, N))
    for i in range(N):
        for j in range(max(0, i - kb), min(N, i + kb + 1)):
            H[i, j] = h0[j * b + (kb + i - j)]
            S[i, j] = repr_.overlap_rows[i, kb + j - i]
    w, v = sl.eigh(H.real, S)
    psi = np.zeros((nang, N), dtype=complex)
    psi[0] = v[:, 0] / np.sqrt(v[:, 0] @ S @ v[:, 0])
    return psi, w[0]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [l.split(", ") for l in self.lines if l.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def l2_flush_buffer(torch):
    return torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _time_launches(torch, fn, flush, reps):
    """Average device time of fn() (CUDA events on the launching stream, L2 flushed before
    every launch unless flush is None, 3 untimed launches first)."""
    stream = torch.cuda.current_stream()
    for _ in range(3):
        fn()
    total = 0.0
    for _ in range(reps):
        if flush is not None:
            flush.fill_(1.0)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        e.synchronize()
        total += s.elapsed_time(e) * 1e-3
    return total / reps


def time_matvec(torch, prob, flush, reps=50):
    """Average duration of the complex64 H matvec kernel and its algorithmic bytes per launch
    s (sum_t P_t + 2 N_psi), s = 8."""
    from pyprop_gb300 import _native as nat
    bp = prob.Propagator.BasePropagator
    op = bp.device_operator(nat.PG_FP32)
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    src = torch.randn((nang, N), dtype=torch.complex64, device="cuda")
    dst = torch.empty_like(src)
    sc = op.scales(5.0)
    avg = _time_launches(torch, lambda: op.matvec(sc, src, dst), flush, reps)
    elems = op.stored_elements()
    return avg, 8 * (elems + 2 * nang * N), op.variant()[0]


def algorithmic_step_bytes(prob, iters, passes):
    """Algorithmic bytes of one mixed step by the per-unit figures of the reference's algorithm:
    per complex64 product of H s (sum_t P_t + 2 N_psi) with s = 8 (P_t = angular pairs x N (2k-1)
    stored band elements of the reference layout), per FP64 product the same with s = 16, per
    block-diagonal solve the LAPACK band LU factors (zgbtrs reads N (3 kb + 1) complex64 values per
    channel) plus the vector in and out, per GMRES iteration j the two classical Gram-Schmidt
    passes 2 (2 j + 2) s N_psi. Solves: one per iteration and per pass; complex64 products one
    per iteration; FP64 products one per pass and one more (the first residual)."""
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    kb = prob.Propagator.op64.kb
    n = nang * N
    P = sum(len(p.PotentialData) * N * (2 * kb + 1) for p in prob.Propagator.BasePropagator.PotentialList)
    mv32 = 8 * (P + 2 * n)
    mv64 = 16 * (P + 2 * n)
    solve = 8 * (nang * N * (3 * kb + 1) + 2 * n)
    full = int(iters)
    cgs = sum(2 * (2 * j + 2) * 8 * n for j in range(full)) + (iters - full) * 2 * (2 * full + 2) * 8 * n
    return int((iters + passes) * solve + iters * mv32 + (passes + 1) * mv64 + cgs)


def step_bytes(prob, iters, passes):
    """Bytes that this implementation's data layout moves in one mixed step (for comparison with
    the algorithmic figure): every block solve reads the dense inverse diagonal blocks, the
    couplings and the boundary inverse (complex64), every complex64 matvec the real FP32 bands
    and its vectors, every FP64 residual product the real FP64 bands and its vectors; the
    solves are one per GMRES iteration and refinement pass, the complex64 products one per
    iteration, the FP64 products one per pass plus the first."""
    from pyprop_gb300 import _native as nat
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    kb = prob.Propagator.op64.kb
    n = nang * N
    nblk = (N + 31) // 32
    per_sweep = nblk * (32 * 32 + 32 * kb) + kb * kb * nblk * (nblk + 1) // 2
    solve = 8 * (nang * 2 * per_sweep + 2 * n)
    e32 = prob.Propagator.opb.stored_elements()
    e64 = prob.Propagator.op64.stored_elements()
    mv32 = 4 * e32 + 8 * 2 * n
    mv64 = 8 * e64 + 16 * 2 * n
    return int((iters + passes) * solve + iters * mv32 + (passes + 1) * mv64)


def time_block_solve(torch, prob, flush, reps=50):
    """Average duration of the complex64 block-diagonal LU solve (both sweeps, one launch) and
    its algorithmic bytes: per fibre and sweep the inverse diagonal blocks (nblk 32x32), the
    couplings (nblk 32 x k) and the nonzero block-triangular half of the boundary inverse
    (k^2 nblk (nblk+1)/2), complex64; plus the fibre read and written."""
    from pyprop_gb300 import _native as nat
    pre = prob.Propagator.Preconditioner.solvers[nat.PG_FP32]
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    kb = prob.Propagator.op64.kb
    x = torch.randn((nang, N), dtype=torch.complex64, device="cuda")
    avg = _time_launches(torch, lambda: pre.apply(nat.PG_BAND_PREC_SOLVE, x), flush, reps)
    nblk = (N + 31) // 32
    per_sweep = nblk * (32 * 32 + 32 * kb) + kb * kb * nblk * (nblk + 1) // 2
    return avg, 8 * (nang * 2 * per_sweep + 2 * nang * N)


LARGE = dict(lmax=300, nbsplines=2000, rmax=2000.0)


MATVEC_KERNELS = {1: "op_matvec_bulk_kernel<float,6,64,false>", 2: "op_matvec_bulk_kernel<float,6,128,false>",
                  3: "op_matvec_kernel<float,6>", 4: "op_matvec_bulk_kernel<float,6,64,true> (TMA)",
                  5: "op_matvec_tma_persistent_kernel<float,6>", 6: "op_matvec_bulk_kernel<float,6,64,rowmajor>",
                  7: "op_matvec_bulk_kernel<float,6,64,true,2> (TMA, 2-block groups)",
                  8: "op_matvec_bulk_kernel<float,6,64,true,1> (TMA, 1-block groups)"}


def time_large_matvec(torch, flush, reps=20):
    """The fused complex64 matvec on an operator larger than L2 (hydrogen lmax 300, 2000
    B-splines: 901 band blocks, 187 MB), where it is HBM-bound: (avg s, algorithmic bytes)."""
    import pyprop_gb300 as pp
    from pyprop_gb300 import _native as nat
    from pyprop_gb300.workloads import hydrogen
    prob = pp.Problem(pp.LoadString(hydrogen(propagator="PamPropagatorGPU", **LARGE)))
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    op = bp.device_operator(nat.PG_FP32)
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    src = torch.randn((nang, N), dtype=torch.complex64, device="cuda")
    dst = torch.empty_like(src)
    sc = op.scales(5.0)
    # the operator (197 MB) is larger than L2: no flush; the launches run back to back between
    # one pair of events (steady-state duration per launch)
    stream = torch.cuda.current_stream()
    for _ in range(3):
        op.matvec(sc, src, dst)
    s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s_ev.record(stream)
    for _ in range(reps):
        op.matvec(sc, src, dst)
    e_ev.record(stream)
    e_ev.synchronize()
    avg = s_ev.elapsed_time(e_ev) * 1e-3 / reps
    nbytes = 8 * (op.stored_elements() + 2 * nang * N)
    variant = op.variant()
    del op, bp, prob
    return avg, nbytes, variant


def profile_large_matvec():
    """Profiling entry point: the large-operator matvec (hydrogen lmax 300, 2000 B-splines)
    after its autotuning, 3 launches inside the NVTX range "matvec_hbm" (for
    ncu --nvtx --nvtx-include matvec_hbm/)."""
    import torch
    import pyprop_gb300 as pp
    from pyprop_gb300 import _native as nat
    from pyprop_gb300.workloads import hydrogen
    prob = pp.Problem(pp.LoadString(hydrogen(propagator="PamPropagatorGPU", **LARGE)))
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    op = bp.device_operator(nat.PG_FP32)
    nang, N = prob.psi.GetRepresentation().GetFullShape()
    src = torch.randn((nang, N), dtype=torch.complex64, device="cuda")
    dst = torch.empty_like(src)
    sc = op.scales(5.0)
    op.matvec(sc, src, dst)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("matvec_hbm")
    for _ in range(3):
        op.matvec(sc, src, dst)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    print(json.dumps({"profile": "matvec_hbm", "variant": MATVEC_KERNELS[op.variant()[0]],
                      "algorithmic_bytes": 8 * (op.stored_elements() + 2 * nang * N)}))


TWO_ELECTRON = dict(lmax=10, L=tuple(range(6)), nbsplines=80, rmax=40.0)


def _two_electron_operator(precision):
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import helium
    prob = pp.Problem(pp.LoadString(helium(**TWO_ELECTRON)))
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    return prob, bp.device_operator(precision)


def time_two_electron(torch, reps=5):
    """The factorized two-electron Hamiltonian (coupled channels L <= 5, l1, l2 <= 10, 80
    B-splines per electron: 291 channels, 1.86e6 coefficients; repulsion multipoles l3 <= 20
    and the field-free terms as angular coefficients x radial band x band operators) applied
    in complex64: (avg s per matvec, flops per matvec, info). The per-factor scratch (> L2)
    makes a flush unnecessary; launches run back to back between one pair of events."""
    from pyprop_gb300 import _native as nat
    t0 = time.perf_counter()
    prob, op = _two_electron_operator(nat.PG_FP32)
    setup = time.perf_counter() - t0
    shape = prob.psi.GetRepresentation().GetFullShape()
    src = torch.randn(shape, dtype=torch.complex64, device="cuda")
    dst = torch.zeros_like(src)
    sc = op.scales(0.0)
    stream = torch.cuda.current_stream()
    for _ in range(2):
        op.matvec(sc, src, dst)
    s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s_ev.record(stream)
    for _ in range(reps):
        op.matvec(sc, src, dst)
    e_ev.record(stream)
    e_ev.synchronize()
    avg = s_ev.elapsed_time(e_ev) * 1e-3 / reps
    info = op.factored_info()
    info["setup_s"] = setup
    info["shape"] = list(shape)
    del op, prob
    return avg, info["flops_mix"] + info["flops_radial"], info


def time_two_electron_steps(torch, steps=3, warmup=1):
    """Cayley steps of the two-electron model of time_two_electron (complex64 matvec with FP64
    refinement, against the plain FP64 path), fast-diagonalization radial preconditioner, a
    length-gauge field on: (dict of steps/s, GMRES iterations, infidelity between the paths)."""
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import helium
    out, states = {}, {}
    psi0 = None
    for prec in ("fp32", "fp64"):
        prob = pp.Problem(pp.LoadString(helium(propagator="CayleyPropagatorGPU", precision=prec, amplitude=0.05,
                                               frequency=0.5, pulse_duration=20.0, duration=20.0, timestep=0.01,
                                               **TWO_ELECTRON)))
        prob.SetupStep(skipWavefunctionSetup=True)
        shape = prob.psi.GetRepresentation().GetFullShape()
        if psi0 is None:
            rng = np.random.default_rng(1)
            decay = np.exp(-0.1 * np.arange(shape[1]))
            psi0 = np.zeros(shape, complex)
            psi0[0] = rng.standard_normal(shape[1:]) * decay[:, None] * decay[None, :]
            psi0 /= np.linalg.norm(psi0)
        prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
        prob.PropagatedTime = 1.0
        for _ in range(warmup):
            prob.AdvanceStep()
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream()
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        iters = 0
        s_ev.record(stream)
        for _ in range(steps):
            prob.AdvanceStep()
            iters += prob.Propagator.LastStats.Iterations
        e_ev.record(stream)
        e_ev.synchronize()
        out[prec] = {"steps_per_s": steps / (s_ev.elapsed_time(e_ev) * 1e-3), "gmres_iterations_per_step": iters / steps,
                     "preconditioner": prob.Propagator.Preconditioner.Method}
        states[prec] = prob.psi.numpy()
        del prob
    a, b = states["fp32"], states["fp64"]
    out["infidelity_mixed_vs_fp64"] = float(1.0 - abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real))
    out["speedup_mixed_vs_fp64"] = out["fp32"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    out["steps"] = steps
    return out


def profile_two_electron():
    """Profiling entry point: the two-electron model of time_two_electron set up for mixed
    Cayley steps; five complex64 matvecs of its operator (overlap slot + factorized terms),
    three solves of its fast-diagonalization preconditioner, three matvecs of its FP64 residual
    operator (factorized terms in double-float)."""
    import torch
    import pyprop_gb300 as pp
    from pyprop_gb300 import _native as nat
    from pyprop_gb300.workloads import helium
    prob = pp.Problem(pp.LoadString(helium(propagator="CayleyPropagatorGPU", precision="fp32", **TWO_ELECTRON)))
    prob.SetupStep(skipWavefunctionSetup=True)
    prop = prob.Propagator
    op = prop.opb
    shape = prob.psi.GetRepresentation().GetFullShape()
    src = torch.randn(shape, dtype=torch.complex64, device="cuda")
    dst = torch.zeros_like(src)
    sc = op.scales(0.0, 0.005j, 1.0)
    for _ in range(5):
        op.matvec(sc, src, dst)
    solver = prop.Preconditioner.solvers[nat.PG_FP32]
    for _ in range(3):
        solver.apply(nat.PG_BAND_PREC_SOLVE, dst)
    # the FP64 residual operator of the mixed step (double-float factorized terms)
    src64 = src.to(torch.complex128)
    dst64 = torch.zeros_like(src64)
    for _ in range(3):
        prop.op64.matvec(sc, src64, dst64)
    torch.cuda.synchronize()
    print(json.dumps({"profile": "two_electron", "info": op.factored_info(),
                      "preconditioner": prop.Preconditioner.Method}))


TWO_ELECTRON_LARGE = dict(lmax=16, L=tuple(range(9)), nbsplines=200, rmax=200.0)


def profile_two_electron_large():
    """Profiling entry point: the largest two-electron model (coupled L <= 8, l1, l2 <= 16, 200
    splines per electron: 1017 channels, 4.07e7 coefficients), three complex64 matvecs of its
    factorized operator after one untimed launch (setup takes about a minute on the host)."""
    import torch
    from pyprop_gb300 import _native as nat
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import helium
    prob = pp.Problem(pp.LoadString(helium(**TWO_ELECTRON_LARGE)))
    bp = prob.Propagator.BasePropagator
    bp.SetupStep(0.01)
    op = bp.device_operator(nat.PG_FP32)
    shape = prob.psi.GetRepresentation().GetFullShape()
    src = torch.randn(shape, dtype=torch.complex64, device="cuda")
    dst = torch.zeros_like(src)
    sc = op.scales(0.0)
    op.matvec(sc, src, dst)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s_ev.record(stream)
    for _ in range(3):
        op.matvec(sc, src, dst)
    e_ev.record(stream)
    e_ev.synchronize()
    info = op.factored_info()
    ms = s_ev.elapsed_time(e_ev) / 3
    print(json.dumps({"profile": "two_electron_large", "ms_per_matvec": ms,
                      "tflops": (info["flops_mix"] + info["flops_radial"]) / ms / 1e9, "info": info}))


def fp32_fma_peak_tflops():
    """Nominal FP32 FMA peak of the GB300 at the maximum SM clock: 152 SMs x 128 lanes x 2 flops
    (no measured FP32 peak exists for this machine)."""
    mhz = 2070.0
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            mhz = float(json.load(fh).get("sm_max_mhz", mhz))
    return 152 * 128 * 2 * mhz * 1e6 / 1e12


def profile_traffic(name):
    """dram bytes per launch recorded in a committed ncu summary (line 'dram_bytes_per_launch: N')."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        for line in fh:
            if line.strip().startswith("dram_bytes_per_launch:"):
                return int(line.split(":")[1].strip())
    return None


def run_ours(args):
    import torch
    import pyprop_gb300 as pp

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    probs = {}
    legs = (("fp32", "fp32", True, None), ("fp64", "fp64", True, None), ("multi", "fp32", False, None),
            ("fp32_tight", "fp32", True, 1e-12), ("fp64_tight", "fp64", True, 1e-12))
    for name, prec, fused, tol in legs:
        p = pp.Problem(pp.LoadString(_config(prec, tol)))
        p.Propagator.StepStats = False  # steps only enqueue; stats are read after the end event
        p.Propagator.Eager = args.eager
        p.Propagator.FusedStep = fused
        p.Propagator.FusedVariant = args.fused_variant
        p.SetupStep(skipWavefunctionSetup=True)
        probs[name] = p
    psi0, e0 = initial_state(probs["fp32"])
    flush = l2_flush_buffer(torch)
    stream = torch.cuda.current_stream()

    def run(prob, K, W, timed=True):
        """W untimed steps, then K steps each bracketed by its own pair of CUDA events on the
        launching stream with the L2 flushed (256 MB write) before it, outside the bracket.
        The steps are enqueued without waiting for each other, so the device timing holds no
        host enqueue latency; returns (device seconds of the K steps, GMRES iterations and
        refinement passes per step, kernels launched)."""
        prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
        prob.PropagatedTime = 0.0
        for _ in range(W):
            prob.AdvanceStep()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        stepper = prob.Propagator.stepper
        ctx = prob.Propagator.op64.ctx
        prob.Propagator.LastStats  # settles the device kernel count of the warm-up steps
        l0 = ctx.launches()
        it0, ps0 = stepper.totals()
        events = []
        for _ in range(K):
            flush.fill_(1.0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            prob.AdvanceStep()
            e.record(stream)
            events.append((s, e))
        torch.cuda.synchronize()
        total = sum(s.elapsed_time(e) for s, e in events) * 1e-3
        it1, ps1 = stepper.totals()
        prob.Propagator.LastStats  # adds this run's device kernel count to the context's
        if dist:
            dist.barrier()
        return total, (it1 - it0) / max(K, 1), (ps1 - ps0) / max(K, 1), ctx.launches() - l0

    with ClockSampler(local) as clk:
        t_mixed, it_mixed, pass_mixed, launches = run(probs["fp32"], args.steps, args.warmup)
    t_fp64, it_fp64, _, _ = run(probs["fp64"], args.steps, args.warmup)
    # the same mixed step on the captured multi-kernel path (comparison only)
    t_multi, it_multi, _, launches_multi = run(probs["multi"], args.steps, args.warmup)
    # both paths at the tight tolerance 1e-12 (comparison only)
    t_mt, it_mt, pass_mt, _ = run(probs["fp32_tight"], args.steps, args.warmup)
    t_dt, it_dt, _, _ = run(probs["fp64_tight"], args.steps, args.warmup)
    fused = bool(getattr(probs["fp32"].Propagator, "Fused", False))
    # 2: the cluster variant (three CTAs per channel), 1: one CTA per channel
    variant = probs["fp32"].Propagator.stepper.fused_variant() if fused else 0
    kernel_name = {2: "cay_cluster_step_kernel<6>", 1: "cay_fused_step_kernel<6>"}.get(variant, "multi-kernel step")
    if dist:
        tt = torch.tensor([t_mixed, t_fp64], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_mixed, t_fp64 = tt.tolist()
    pulse = pulse_against_reference(run, probs, psi0) if args.pulse else None

    # end to end through the public API with host buffers: H2D + step + D2H per step
    prob = probs["fp32"]
    host = torch.empty(psi0.shape, dtype=torch.complex128).pin_memory()
    host.copy_(torch.as_tensor(psi0))
    dev = prob.psi.GetData()
    prob.PropagatedTime = 0.0
    for _ in range(args.warmup):
        dev.copy_(host, non_blocking=True)
        prob.AdvanceStep()
        host.copy_(dev, non_blocking=True)
        torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dev.copy_(host, non_blocking=True)
        prob.AdvanceStep()
        host.copy_(dev, non_blocking=True)
        torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    nbytes = psi0.size * 16

    avg_mv, bytes_mv, variant_mv = time_matvec(torch, prob, flush)
    bytes_step = algorithmic_step_bytes(prob, it_mixed, pass_mixed)
    layout_bytes_step = step_bytes(prob, it_mixed, pass_mixed)
    avg_ts, bytes_ts = time_block_solve(torch, prob, flush)
    avg_lg, bytes_lg, variant_lg = time_large_matvec(torch, flush)
    two_e = time_two_electron(torch) if args.two_electron else None
    two_e_steps = time_two_electron_steps(torch) if args.two_electron else None
    peak, peak_kind = measured_peaks()

    ens = run_ensemble(args, torch, flush) if args.ensemble > 0 else None
    ens_pamp = run_pamp_ensemble(args, torch, flush) if args.ensemble > 0 else None
    two_e_large = time_two_electron_large(torch) if (args.two_electron_large and rank == 0) else None
    learned = time_learned_helium(torch) if (args.learned and rank == 0) else None
    pamp_l10 = time_pamp_hydrogen_l10(torch, flush) if (args.pamp_l10 and rank == 0) else None
    if pamp_l10 is not None and world == 1 and args.cpu_steps > 0:
        pamp_l10["cpu_baseline"] = cpu_pamp_sample()
        pamp_l10["speedup_vs_cpu_port"] = pamp_l10["fp32"]["steps_per_s"] / pamp_l10["cpu_baseline"]["value"]
    cpu = cpu_baseline_sample(nsteps=args.cpu_steps) if (rank == 0 and world == 1 and args.cpu_steps > 0) else None
    if rank == 0:
        steps_per_s = world * args.steps / t_mixed
        line = {
            "metric": METRIC, "value": steps_per_s, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_mixed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 matvec/basis, f64 reductions+residual",
            "data": "synthetic (hydrogen model built from the config; initial state = field-free 1s)",
            "config": {"workload": "hydrogen lmax=40 N=600 rmax=400 Cayley-GMRES(20) block-diag LU, dt=0.01, "
                                   "800nm sin2 pulse 0.05au", "global_batch": world, "seq_len": None,
                       "parallelism": "replicas" if world > 1 else "single", "l2": "flushed before every step"},
            "gmres_tolerance": probs["fp32"].Propagator.Tolerance,
            "plain_fp64": {"steps_per_s": world * args.steps / t_fp64, "gmres_iterations_per_step": it_fp64,
                           "gmres_tolerance": probs["fp64"].Propagator.Tolerance},
            "speedup_vs_plain_fp64": t_fp64 / t_mixed,
            "infidelity_vs_reference": None if pulse is None else pulse["mixed"]["infidelity_vs_reference"],
            "equal_error": pulse,
            "gmres_iterations_per_step": it_mixed,
            "refinement_passes_per_step": pass_mixed,
            "tight_tolerance": {"gmres_tolerance": 1e-12, "mixed_steps_per_s": world * args.steps / t_mt,
                                "mixed_gmres_iterations_per_step": it_mt, "mixed_passes_per_step": pass_mt,
                                "fp64_steps_per_s": world * args.steps / t_dt, "fp64_gmres_iterations_per_step": it_dt,
                                "speedup": t_dt / t_mt},
            "e2e": {"value": world * args.steps / e2e_t, "unit": "steps/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            # dominant kernel: the single-kernel step itself (one launch per step)
            "roofline": {"bound": "hbm", "achieved": bytes_step / (t_mixed / args.steps) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": bytes_step / (t_mixed / args.steps) / 1e9 / peak,
                         # ncu does not keep the cluster variant's launch shape (thread-block clusters in a
                         # cooperative launch), so its DRAM bytes come from the one-CTA-per-channel
                         # variant, which reads the same working set
                         "traffic": profile_traffic("cay_fused_step_kernel_lmax40_n600.md"),
                         "traffic_source": "ncu capture of cay_fused_step_kernel<6> (same step, one CTA per "
                                           "channel, same working set)" if variant == 2 else "ncu capture",
                         "kernel": kernel_name,
                         "avg_launch_us": 1e6 * t_mixed / args.steps, "algorithmic_bytes": bytes_step,
                         "layout_bytes": layout_bytes_step, "peak_kind": peak_kind,
                         "bytes_rule": "per complex64/FP64 product s(sum P_t + 2 N_psi), per block solve the LAPACK "
                                       "band LU factors N(3kb+1) per channel + 2 s N_psi, per iteration CGS2 "
                                       "2(2j+2) s N_psi; layout_bytes = what this implementation's dense block "
                                       "inverses and real bands move",
                         "timing": "CUDA events around each timed step on the launching stream, L2 flushed before each",
                         "note": "block-solve factors and bands are re-read from L2 within a step: latency-bound "
                                 "(grid barriers, dependent block-solve phases), not HBM-bound"},
            "roofline_block_solve": {"bound": "hbm", "achieved": bytes_ts / avg_ts / 1e9, "peak": peak, "unit": "GB/s",
                                     "frac": bytes_ts / avg_ts / 1e9 / peak,
                                     "traffic": profile_traffic("tri_solve_kernel_fp32_lmax40_n600.md"),
                                     "kernel": "tri_solve_kernel<float,cx<float>,24>", "avg_launch_us": 1e6 * avg_ts,
                                     "algorithmic_bytes": bytes_ts, "peak_kind": peak_kind,
                                     "timing": "CUDA events around 50 launches, L2 flushed before each"},
            "multi_kernel_step": {"steps_per_s": world * args.steps / t_multi, "gmres_iterations_per_step": it_multi,
                                  "kernels_per_step": launches_multi / max(args.steps, 1)},
            "roofline_matvec": {"bound": "hbm", "achieved": bytes_mv / avg_mv / 1e9, "peak": peak, "unit": "GB/s",
                                "frac": bytes_mv / avg_mv / 1e9 / peak,
                                "traffic": profile_traffic("op_matvec_bulk_kernel_fp32_lmax40_n600.md"),
                                "kernel": MATVEC_KERNELS[variant_mv], "avg_launch_us": 1e6 * avg_mv,
                                "algorithmic_bytes": bytes_mv,
                                "note": "7.9 MB operator: launch- and latency-bound at this size"},
            "roofline_matvec_hbm": {"bound": "hbm", "achieved": bytes_lg / avg_lg / 1e9, "peak": peak, "unit": "GB/s",
                                    "frac": bytes_lg / avg_lg / 1e9 / peak, "kernel": MATVEC_KERNELS[variant_lg[0]],
                                    "avg_launch_us": 1e6 * avg_lg, "algorithmic_bytes": bytes_lg,
                                    "workload": "hydrogen lmax 300, 2000 B-splines (operator > L2; 20 launches back to back)",
                                    "variant": variant_lg[0], "tuning_us": variant_lg[1]},
            "roofline_two_electron": None if two_e is None else {
                "bound": "fma", "achieved": two_e[1] / two_e[0] / 1e12, "peak": fp32_fma_peak_tflops(),
                "unit": "TFLOP/s", "frac": two_e[1] / two_e[0] / 1e12 / fp32_fma_peak_tflops(),
                "peak_kind": "nominal FP32 FMA peak at the maximum SM clock (no measured FP32 peak)",
                "kernels": "fact_mix_kernel<float> + fact_radial_kernel<float,6,128,32,8,4>",
                "ms_per_matvec": 1e3 * two_e[0], "flops_per_matvec": two_e[1],
                "workload": "helium-like, coupled L<=5, l1,l2<=10, 80 B-splines per electron (rank 3, factorized "
                            "repulsion multipoles + field-free terms), complex64, 5 launches back to back",
                "info": two_e[2]},
            "two_electron_cayley": two_e_steps,
            "two_electron_large": two_e_large,
            "learned_helium": learned,
            "pamp_hydrogen_l10": pamp_l10,
            "cpu_baseline": cpu,
            "ensemble": ens,
            "ensemble_pamp": ens_pamp,
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "ground_energy": e0,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def _rank_world():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def _my_members(n):
    """This rank's share of the ensemble's member parameters (replicas only: each rank steps
    its own contiguous range, no collective on the data path)."""
    from pyprop_gb300.ensemble import hydrogen_ensemble_params, partition_members
    rank, world = _rank_world()
    a, b = partition_members(n, world, rank)
    return hydrogen_ensemble_params(n)[a:b]


def pulse_against_reference(run, probs, psi0):
    """The whole 5000-step pulse on the mixed and the plain FP64 path at their equal-error
    tolerances (steps timed as in the headline: CUDA events per step, L2 flushed before each),
    each final state against the complex128 reference run: S-weighted infidelity, S-norm and
    energy differences. None when the reference run's fixture is absent."""
    if not os.path.exists(REFERENCE_RUN):
        return None
    from pyprop_gb300.workloads import run_steps
    g = np.load(REFERENCE_RUN)
    kw = dict(WORKLOAD, duration=50.0)
    nsteps = run_steps(kw)
    if np.max(np.abs(g["psi0"] - psi0)) > 1e-12:
        raise RuntimeError("the reference run starts from another initial state")
    out = {"bar": 1e-8, "steps": nsteps, "reference": "tests/golden/run_cayley_l40.npz (complex128, the "
           "reference's own GMRES template, GMRES tolerance 1e-12)"}
    for name, key in (("mixed", "fp32"), ("fp64", "fp64")):
        prob = probs[key]
        t, it, ps, _ = run(prob, nsteps, 0)
        psi = prob.psi.numpy()
        repr_ = prob.psi.GetRepresentation()
        S = repr_.radial.BSplineObject.dense(repr_.overlap_rows)
        Sp = psi @ S.T
        r = psi - g["psi"] * (np.vdot(g["psi"], Sp) / np.vdot(g["psi"], g["psi"] @ S.T).real)
        out[name] = {"gmres_tolerance": prob.Propagator.Tolerance, "pulse_steps_per_s": nsteps / t,
                     "infidelity_vs_reference": float(np.vdot(r, r @ S.T).real / np.vdot(psi, Sp).real),
                     "norm_error": abs(prob.psi.GetNorm() - float(g["norm"])),
                     "energy_error": abs(prob.GetEnergyExpectationValue() - float(g["energy"])),
                     "gmres_iterations_per_step": it, "refinement_passes_per_step": ps}
    out["speedup"] = out["mixed"]["pulse_steps_per_s"] / out["fp64"]["pulse_steps_per_s"]
    return out


def run_ensemble(args, torch, flush):
    """Batched ensemble: member-steps/s of one graph launch per ensemble step (mixed
    precision), against the same members stepped one at a time on the plain FP64 path. With
    several ranks each steps its share of the members; the job rate is the member steps of
    all ranks over the slowest rank's time."""
    import pyprop_gb300 as pp
    from pyprop_gb300.ensemble import CayleyEnsembleGPU, job_throughput
    from pyprop_gb300.workloads import hydrogen
    t_setup = time.perf_counter()
    params = _my_members(args.ensemble)

    def member(prm, precision):
        p = pp.Problem(pp.LoadString(hydrogen(propagator="CayleyPropagatorGPU", precision=precision, rmax=100.0,
                                              timestep=0.01, pulse_duration=10.0, duration=10.0,
                                              krylov_basis_size=20, gmres_tolerance=1e-12, **prm)))
        p.Propagator.StepStats = False
        p.SetupStep(skipWavefunctionSetup=True)
        psi, _ = initial_state(p)
        p.psi.SetData(psi)
        return p, psi

    members = [member(prm, "fp32") for prm in params]
    probs = [m[0] for m in members]
    ens = CayleyEnsembleGPU(probs)
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        ens.AdvanceStep()
    torch.cuda.synchronize()
    K = max(1, min(args.steps, 20))
    table = ens.scale_table(K)
    stream = torch.cuda.current_stream()
    total = 0.0
    iters = 0
    for k in range(K):
        flush.fill_(1.0)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        ens.AdvanceStep(table[k])
        e.record(stream)
        e.synchronize()
        total += s.elapsed_time(e) * 1e-3
        iters += sum(st["Iterations"] for st in ens.Stats())
    member_steps = K * len(probs)
    # plain FP64 path on a sample of the same members, one member step at a time
    sample = list(range(0, len(params), max(1, len(params) // 16)))[:16]
    t64 = 0.0
    n64 = 0
    for i in sample:
        p64, psi = member(params[i], "fp64")
        for _ in range(3):
            p64.AdvanceStep()
        torch.cuda.synchronize()
        for _ in range(5):
            flush.fill_(1.0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            p64.AdvanceStep()
            e.record(stream)
            e.synchronize()
            t64 += s.elapsed_time(e) * 1e-3
            n64 += 1
        del p64
    fp64_rate = n64 / t64
    rate, _, t_job = job_throughput(member_steps, total, _rank_world()[1])
    return {"members": args.ensemble, "member_steps_per_s": rate, "ms_per_ensemble_step": 1e3 * t_job / K,
            "gmres_iterations_per_member_step": iters / member_steps,
            "plain_fp64_single_member_steps_per_s": fp64_rate, "speedup_vs_plain_fp64": rate / fp64_rate,
            "workload": "%d hydrogen members, lmax U{8..32}, N U{100..400} on r in [0,100], E0 U[0.01,0.1], "
                        "lambda U[400,1600] nm (rng seed 20261203), Cayley mixed precision, one graph launch per "
                        "ensemble step, L2 flushed between steps" % len(probs),
            "setup_s": setup_s}


def pamp_member_bytes(prob, m):
    """Algorithmic bytes of one pAMP step of a member at complex64 (s = 8): m (B_mv + 2 B_S) +
    sum_j B_GS(j), with B_mv = s (sum_t P_t + 2 N_psi) (P_t: stored elements of term t in the
    reference's TensorPotential layout), B_S = 2 s N_psi per overlap solve (two per matvec in
    the balanced form), B_GS(j) = 2 (2j + 2) s N_psi for CGS2 against j + 1 vectors."""
    s = 8
    n = int(np.prod(prob.psi.GetRepresentation().GetFullShape()))
    P = sum(int(np.asarray(pot.PotentialData).size) for pot in prob.Propagator.BasePropagator.PotentialList)
    b_mv = s * (P + 2 * n)
    b_s = 2 * s * n
    return m * (b_mv + 2 * b_s) + sum(2 * (2 * j + 2) * s * n for j in range(m))


def _pamp_members(params, precision):
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import hydrogen
    out = []
    for prm in params:
        p = pp.Problem(pp.LoadString(hydrogen(propagator="PamPropagatorGPU", precision=precision, rmax=100.0,
                                              timestep=0.01, pulse_duration=10.0, duration=10.0,
                                              krylov_basis_size=20, **prm)))
        p.SetupStep(skipWavefunctionSetup=True)
        psi, _ = initial_state(p)
        p.psi.SetData(psi)
        out.append(p)
    return out


def _time_ensemble(torch, flush, ens, probs, K):
    """Device seconds of K ensemble steps (CUDA events around each, L2 flushed before each
    outside the bracket), slot values of each step precomputed."""
    tables = [np.stack([p.Propagator.op64.scales(p.PropagatedTime + k * ens.dt) for p in probs]) for k in range(K)]
    stream = torch.cuda.current_stream()
    total = 0.0
    for k in range(K):
        flush.fill_(1.0)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        ens.AdvanceStep(tables[k])
        e.record(stream)
        e.synchronize()
        total += s.elapsed_time(e) * 1e-3
    return total


def run_pamp_ensemble(args, torch, flush):
    """The ensemble of run_ensemble with pAMP steps (Krylov basis 20, complex64 basis with FP64
    Gram-Schmidt sums, the m x m exponentials of all members on the device). The step is the
    faster of the persistent kernel (one launch per ensemble step, one CTA per member from a
    device work list) and the graph of every member's kernels, as the batch's autotuner picks
    it at its first step; both times are reported. Compared with the same members batched on a
    complex128 basis (the graph: the persistent kernel takes complex64 bases) and one at a time
    on the plain FP64 pAMP path (host exponential)."""
    from pyprop_gb300.ensemble import PamEnsembleGPU, job_throughput
    t_setup = time.perf_counter()
    params = _my_members(args.ensemble)
    probs = _pamp_members(params, "fp32")
    ens = PamEnsembleGPU(probs)
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        ens.AdvanceStep()
    torch.cuda.synchronize()
    K = max(1, min(args.steps, 20))
    total = _time_ensemble(torch, flush, ens, probs, K)
    shape = ens.launch_shape()
    err = max(st["ErrorEstimate"] for st in ens.Stats())
    member_steps = K * len(probs)
    bytes_step = sum(pamp_member_bytes(p, 20) for p in probs)
    del ens
    # the same members batched on a complex128 basis (one graph launch per ensemble step)
    p64 = _pamp_members(params, "fp64")
    e64 = PamEnsembleGPU(p64)
    for _ in range(2):
        e64.AdvanceStep()
    torch.cuda.synchronize()
    K64 = max(1, min(K, 5))
    t64b = _time_ensemble(torch, flush, e64, p64, K64)
    del e64
    # and one member at a time on the plain FP64 path, on a sample of the members
    sample = list(range(0, len(params), max(1, len(params) // 16)))[:16]
    stream = torch.cuda.current_stream()
    t64 = 0.0
    n64 = 0
    for i in sample:
        q = p64[i]
        for _ in range(3):
            q.AdvanceStep()
        torch.cuda.synchronize()
        for _ in range(5):
            flush.fill_(1.0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            q.AdvanceStep()
            e.record(stream)
            e.synchronize()
            t64 += s.elapsed_time(e) * 1e-3
            n64 += 1
    del p64
    fp64_rate = n64 / t64
    world = _rank_world()[1]
    rate, _, t_job = job_throughput(member_steps, total, world)
    rate64b, _, _ = job_throughput(K64 * len(probs), t64b, world)
    peak, peak_kind = measured_peaks()
    achieved = bytes_step / (total / K) / 1e9
    return {"members": args.ensemble, "member_steps_per_s": rate, "ms_per_ensemble_step": 1e3 * t_job / K,
            "step": "persistent kernel" if shape["persistent"] else "graph of per-member kernels",
            "autotuned": shape, "max_error_estimate": err,
            "batched_fp64_member_steps_per_s": rate64b, "speedup_vs_batched_fp64": rate / rate64b,
            "plain_fp64_single_member_steps_per_s": fp64_rate, "speedup_vs_plain_fp64": rate / fp64_rate,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "algorithmic_bytes": bytes_step, "peak_kind": peak_kind,
                         "traffic": profile_traffic("pm_step_kernel_pamp_ensemble256.md"),
                         "kernel": "pm_step_kernel (persistent)" if shape["persistent"] else "graph",
                         "bytes_rule": "per member m (B_mv + 2 B_S) + sum_j B_GS(j), complex64"},
            "workload": "the members of `ensemble` with pAMP (m=20, complex64 basis, FP64 sums), one launch per "
                        "ensemble step including the device Pade exponentials, L2 flushed between steps",
            "setup_s": setup_s}


def time_two_electron_large(torch, steps=2):
    """The largest two-electron model (coupled L <= 8, l1, l2 <= 16, 200 B-splines of order 7
    per electron on r in [0, 200]: 1017 channels, 4.07e7 coefficients) end to end: operator
    set-up (two-electron radial factors projected on the GPU), then mixed-precision Cayley
    steps (complex64 factorized matvec, FP64 refinement in double-float, fast-diagonalization
    radial preconditioner) in a length-gauge field; one untimed step first."""
    import pyprop_gb300 as pp
    from pyprop_gb300 import _native as nat
    from pyprop_gb300.workloads import helium
    t0 = time.perf_counter()
    prob = pp.Problem(pp.LoadString(helium(propagator="CayleyPropagatorGPU", precision="fp32", amplitude=0.05,
                                           frequency=0.5, pulse_duration=20.0, duration=20.0, timestep=0.01,
                                           **TWO_ELECTRON_LARGE)))
    prob.SetupStep(skipWavefunctionSetup=True)
    setup_s = time.perf_counter() - t0
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(1)
    decay = np.exp(-0.05 * np.arange(shape[1]))
    psi0 = np.zeros(shape, complex)
    psi0[0] = rng.standard_normal(shape[1:]) * decay[:, None] * decay[None, :]
    psi0 /= np.linalg.norm(psi0)
    prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
    prob.PropagatedTime = 1.0
    prob.AdvanceStep()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters = 0
    resid = 0.0
    s_ev.record(stream)
    for _ in range(steps):
        prob.AdvanceStep()
        st = prob.Propagator.LastStats
        iters += st.Iterations
        resid = max(resid, st.TrueResidual)
    e_ev.record(stream)
    e_ev.synchronize()
    step_s = s_ev.elapsed_time(e_ev) * 1e-3 / steps
    # the complex64 matvec of the factorized operator alone
    op = prob.Propagator.BasePropagator.device_operator(nat.PG_FP32)
    src = torch.randn(tuple(shape), dtype=torch.complex64, device="cuda")
    dst = torch.zeros_like(src)
    sc = op.scales(1.0)
    op.matvec(sc, src, dst)
    torch.cuda.synchronize()
    s_ev.record(stream)
    for _ in range(3):
        op.matvec(sc, src, dst)
    e_ev.record(stream)
    e_ev.synchronize()
    ms = s_ev.elapsed_time(e_ev) / 3
    info = op.factored_info()
    flops = info["flops_mix"] + info["flops_radial"]
    peak = fp32_fma_peak_tflops()
    return {"workload": "helium-like, coupled L<=8, l1,l2<=16, 200 B-splines order 7 per electron, r in [0,200] "
                        "(1017 channels, %d coefficients), Cayley GMRES(20) mixed precision, fast-diagonalization "
                        "preconditioner, dt=0.01, field on" % int(np.prod(shape)),
            "setup_s": setup_s, "steps": steps, "steps_per_s": 1.0 / step_s, "s_per_step": step_s,
            "gmres_iterations_per_step": iters / steps, "fp64_true_residual": resid,
            "norm": prob.psi.GetNorm(),
            "roofline_matvec": {"bound": "fma", "achieved": flops / ms / 1e9, "peak": peak, "unit": "TFLOP/s",
                                "frac": flops / ms / 1e9 / peak, "ms_per_matvec": ms,
                                "peak_kind": "nominal FP32 FMA peak at the maximum SM clock"},
            "parity": "oracle comparison at reduced size with the same code path: tests/test_gpu_helium.py"}


def time_pamp_hydrogen_l10(torch, flush, steps=1000, warmup=5):
    """Hydrogen lmax 10, 150 B-splines, rmax 100, pAMP with 20 Krylov vectors, dt 0.01 through
    the 10 a.u. 800 nm pulse (1000 steps), from the field-free 1s state: steps per second of the
    single-wavefunction step: complex64 basis as one cooperative kernel per step (the default)
    and as captured graphs; complex128 basis as graphs with the m x m exponential on the host
    between them (the default: FP64 arithmetic is scarce on this GPU) and on the device. CUDA
    events around each step on the launching stream, L2 flushed (256 MB write) before each,
    outside the bracket."""
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import HYDROGEN_L10_PAMP, hydrogen
    stream = torch.cuda.current_stream()
    out = {"workload": "hydrogen lmax=10 N=150 rmax=100 pAMP(20), dt=0.01, 800nm sin2 pulse 0.05au, 1000 steps",
           "timing": "CUDA events around each step, L2 flushed before each"}
    psi0 = None
    for name, prec, fused, dev in (("fp32", "fp32", True, False), ("fp32_graphs", "fp32", False, False),
                                   ("fp64", "fp64", False, False), ("fp64_device_exp", "fp64", False, True)):
        prob = pp.Problem(pp.LoadString(hydrogen(propagator="PamPropagatorGPU", precision=prec, **HYDROGEN_L10_PAMP)))
        prob.SetupStep(skipWavefunctionSetup=True)
        if prob.Propagator.stepper.set_fused(fused) != fused:
            raise RuntimeError("pAMP leg: the single-kernel step does not take this workload")
        prob.Propagator.stepper.set_device_exp(dev)
        prob.Propagator.StepStats = False
        if psi0 is None:
            psi0, _ = initial_state(prob)
        prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
        prob.PropagatedTime = 0.0
        ctx = prob.Propagator.op64.ctx
        for _ in range(warmup):
            prob.AdvanceStep()
        torch.cuda.synchronize()
        prob.PropagatedTime = 0.0
        prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
        l0 = ctx.launches()
        events = []
        for _ in range(steps):
            flush.fill_(1.0)
            s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s_ev.record(stream)
            prob.AdvanceStep()
            e_ev.record(stream)
            events.append((s_ev, e_ev))
        torch.cuda.synchronize()
        total = sum(a.elapsed_time(b) for a, b in events) * 1e-3
        st = prob.Propagator.LastStats
        if name == "fp32":
            prob_fused = prob
        out[name] = {"steps_per_s": steps / total, "us_per_step": 1e6 * total / steps,
                     "kernels_per_step": (ctx.launches() - l0) / steps, "norm_after_pulse": prob.psi.GetNorm(),
                     "error_estimate_last_step": st.ErrorEstimate}
    # the single-kernel step's roofline: algorithmic bytes of one complex64-basis step
    peak, peak_kind = measured_peaks()
    nbytes = pamp_member_bytes(prob_fused, 20)
    ach = nbytes / (out["fp32"]["us_per_step"] * 1e-6) / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                       "traffic": profile_traffic("pamp_fused_step_kernel_hydrogen_l10_n150.md"),
                       "kernel": "pamp_fused_step_kernel<6,2>", "algorithmic_bytes": nbytes, "peak_kind": peak_kind,
                       "note": "1.3 MB working set resident in L2 and shared memory: latency-bound (grid and CTA "
                               "barriers)"}
    out["single_kernel_speedup_vs_graphs"] = out["fp32"]["steps_per_s"] / out["fp32_graphs"]["steps_per_s"]
    out["speedup_vs_plain_fp64"] = out["fp32"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    out["parity"] = ("tests/test_gpu_parity.py: the whole pulse (40 vectors) and the first steps (20 vectors) against "
                     "the reference templates' states")
    return out


def time_learned_helium(torch):
    """The learned preconditioner at the helium model of TWO_ELECTRON (coupled L <= 5, l1, l2
    <= 10, 80 B-splines per electron: 291 angular blocks of 6400 coefficients), field free, on
    top of the fast-diagonalization block preconditioner; the network learns the part of the
    correction the blocks miss (the electron-electron repulsion). 172 harvested steps give
    50 052 (residual, correction) block pairs (85% train, 15% held out); 3000 Adam steps on
    the GPU; then 20 Cayley steps with and without the network from the same state."""
    import pyprop_gb300 as pp
    from pyprop_gb300.learned import LearnedPreconditioner
    from pyprop_gb300.workloads import helium
    prob = pp.Problem(pp.LoadString(helium(propagator="CayleyPropagatorGPU", precision="fp32", amplitude=0.0,
                                           timestep=0.01, duration=20.0, gmres_tolerance=1e-10, **TWO_ELECTRON)))
    prob.SetupStep(skipWavefunctionSetup=True)
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(1)
    decay = np.exp(-0.1 * np.arange(shape[1]))
    psi0 = np.zeros(shape, complex)
    psi0[0] = rng.standard_normal(shape[1:]) * decay[:, None] * decay[None, :]
    psi0 /= np.linalg.norm(psi0)
    prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
    prob.PropagatedTime = 1.0
    pots = prob.Propagator.BasePropagator.PotentialList
    rep = [k for k, pot in enumerate(pots) if "ElectronicCoupling" in getattr(pot, "Name", "")][0]
    lp = LearnedPreconditioner(prob.Propagator, hidden=256, coupling_potential=rep)
    t0 = time.perf_counter()
    lp.harvest(prob, 172)
    ntr = int(0.85 * len(lp.pairs))
    X, T = lp.training_set(lp.pairs[:ntr])
    t1 = time.perf_counter()
    losses = lp.train(X, T, steps=3000, lr=3e-4, batch=1024)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    rows = int(X.shape[0])
    del X, T
    held = lp.pairs[ntr:]
    out = {"workload": "helium-like, coupled L<=5, l1,l2<=10, 80 B-splines per electron (291 blocks of 6400), "
                       "field free, fast-diagonalization blocks + learned correction of the repulsion",
           "network": "%d -> 256 -> 256 -> %d, %d parameters (BF16 weights, FP32 accumulate)" %
                      (lp.d_in, lp.d_out, lp.net.parameter_count()),
           "pairs": len(lp.pairs) * shape[0], "training_rows": rows, "train_s": t_train,
           "harvest_s": t1 - t0, "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
           "held_out_one_step_residual": {"block": lp.one_step_residual(held, learned=False),
                                          "learned": lp.one_step_residual(held, learned=True)}}
    out.update(lp.compare_steps(prob, 20))
    return out


def profile_ensemble_pamp():
    """Profiling entry point: the 256-member pAMP ensemble on the persistent kernel (forced),
    its autotuning launches at the first step, then three steps."""
    import torch
    from pyprop_gb300.ensemble import PamEnsembleGPU, hydrogen_ensemble_params
    probs = _pamp_members(hydrogen_ensemble_params(256), "fp32")
    ens = PamEnsembleGPU(probs)
    ens.set_persistent(True)
    for _ in range(4):
        ens.AdvanceStep()
    torch.cuda.synchronize()
    print(json.dumps({"profile": "ensemble_pamp", "shape": ens.launch_shape()}))


def profile_pamp_l10():
    """Profiling entry point: the single-wavefunction pAMP workload (hydrogen lmax 10, 150
    B-splines, basis 20, complex64) on the single-kernel step, 7 steps from the 1s state."""
    import torch
    import pyprop_gb300 as pp
    from pyprop_gb300.workloads import HYDROGEN_L10_PAMP, hydrogen
    prob = pp.Problem(pp.LoadString(hydrogen(propagator="PamPropagatorGPU", precision="fp32", **HYDROGEN_L10_PAMP)))
    prob.SetupStep(skipWavefunctionSetup=True)
    prob.Propagator.StepStats = False
    psi0, _ = initial_state(prob)
    prob.psi.GetData().copy_(torch.as_tensor(psi0, device="cuda"))
    for _ in range(7):
        prob.AdvanceStep()
    torch.cuda.synchronize()
    print(json.dumps({"profile": "pamp_l10", "fused": bool(prob.Propagator.Fused), "norm": prob.psi.GetNorm()}))


# ---------------------------------------------------------------------------------------
# CPU reference (oracle port of the reference algorithm)
# ---------------------------------------------------------------------------------------

def _oracle_setup():
    import pyprop_gb300 as pp
    from oracle.propagators import OracleCayley, OracleHamiltonian
    prob = pp.Problem(pp.LoadString(_config("fp64")))
    repr_ = prob.psi.GetRepresentation()
    nang, N = repr_.GetFullShape()
    bp = prob.Propagator.BasePropagator
    terms = [("_".join(g.GetStorageId() for g in p.GeometryList), p.PotentialData, p.GeometryList[0].GetBasisPairs(),
              p.TimeFunction) for p in bp.PotentialList]
    ham = OracleHamiltonian(terms, repr_.overlap_rows, nang, N)
    from pyprop_gb300.workloads import EQUAL_ERROR_TOLERANCE
    # complex128 like the plain FP64 path: the same equal-error GMRES tolerance
    cay = OracleCayley(ham, WORKLOAD["timestep"], [0], WORKLOAD["krylov_basis_size"], EQUAL_ERROR_TOLERANCE["fp64"])
    psi0, _ = initial_state(prob)
    return cay, psi0


def _oracle_worker(nsteps, q):
    cay, psi = _oracle_setup()
    dt = WORKLOAD["timestep"]
    t0 = time.perf_counter()
    t = 0.0
    for _ in range(nsteps):
        psi = cay.step(psi, t, dt)
        t += dt
    q.put(time.perf_counter() - t0)


def cpu_baseline_sample(nsteps=20, procs=1):
    """Oracle Cayley steps on the host, `procs` processes each stepping its own copy."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    # one BLAS thread per process: set before the children start (their numpy reads it at import)
    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in saved:
        os.environ[k] = "1"
    try:
        ps = [ctx.Process(target=_oracle_worker, args=(nsteps, q)) for _ in range(procs)]
        for p in ps:
            p.start()
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    times = [q.get() for _ in ps]
    for p in ps:
        p.join()
    from pyprop_gb300.workloads import EQUAL_ERROR_TOLERANCE
    return {"value": procs * nsteps / max(times), "unit": "steps/s", "cores": procs, "kind": "port",
            "sample": "%d Cayley steps from t=0 per process, numpy/scipy complex128 oracle of the reference "
                      "algorithm at GMRES tolerance %g (the complex128 equal-error tolerance; "
                      "OPENBLAS_NUM_THREADS=1)" % (nsteps, EQUAL_ERROR_TOLERANCE["fp64"])}


def _oracle_pamp_worker(nsteps, q):
    """Oracle pAMP steps (complex128, basis 20, CGS2) of the single-wavefunction pAMP workload."""
    import pyprop_gb300 as pp
    from oracle.propagators import OracleHamiltonian, OraclePam
    from pyprop_gb300.workloads import HYDROGEN_L10_PAMP, hydrogen
    prob = pp.Problem(pp.LoadString(hydrogen(propagator="PamPropagatorGPU", precision="fp64", **HYDROGEN_L10_PAMP)))
    repr_ = prob.psi.GetRepresentation()
    nang, N = repr_.GetFullShape()
    bp = prob.Propagator.BasePropagator
    terms = [("_".join(g.GetStorageId() for g in p.GeometryList), p.PotentialData, p.GeometryList[0].GetBasisPairs(),
              p.TimeFunction) for p in bp.PotentialList]
    pam = OraclePam(OracleHamiltonian(terms, repr_.overlap_rows, nang, N), HYDROGEN_L10_PAMP["krylov_basis_size"], True)
    psi, _ = initial_state(prob)
    dt = HYDROGEN_L10_PAMP["timestep"]
    t0 = time.perf_counter()
    for n in range(nsteps):
        psi = pam.step(psi, n * dt, dt)
    q.put(time.perf_counter() - t0)


def cpu_pamp_sample(nsteps=100):
    """The oracle port of the reference's pAMP step on one host core (spawned process, one BLAS
    thread) for the single-wavefunction pAMP workload."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in saved:
        os.environ[k] = "1"
    try:
        proc = ctx.Process(target=_oracle_pamp_worker, args=(nsteps, q))
        proc.start()
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    elapsed = q.get()
    proc.join()
    return {"value": nsteps / elapsed, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": "%d pAMP steps from the field-free 1s state, numpy/scipy complex128 oracle of the reference "
                      "algorithm (basis 20, CGS2; OPENBLAS_NUM_THREADS=1)" % nsteps}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    nsteps = max(10, min(args.steps, 300))
    base = cpu_baseline_sample(nsteps=nsteps, procs=procs)
    line = {"metric": METRIC, "value": base["value"], "unit": "steps/s", "n_gpus": 0, "steps": nsteps * procs,
            "warmup": 0, "ms_per_step": 1e3 / base["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic", "impl": "reference",
            "config": {"workload": "hydrogen lmax=40 N=600 rmax=400 Cayley-GMRES(20) block-diag LU, dt=0.01"},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=300,
                    help="oracle Cayley steps timed on one host core for cpu_baseline (0 = skip)")
    ap.add_argument("--two-electron", type=int, default=1, help="factorized two-electron matvec leg (0 = skip)")
    ap.add_argument("--profile", choices=["matvec_hbm", "two_electron", "two_electron_large", "ensemble_pamp", "pamp_l10"],
                    default=None, help="profiling entry point instead of the benchmark")
    ap.add_argument("--fused-variant", type=int, default=0, choices=[0, 1, 2],
                    help="single-kernel Cayley step layout: 0 the cluster variant where it fits, 1 one CTA per "
                         "channel (the layout to profile: ncu does not keep a cooperative launch's cluster shape), "
                         "2 the cluster variant")
    ap.add_argument("--two-electron-large", type=int, default=1,
                    help="end-to-end leg of the largest two-electron model (0 = skip)")
    ap.add_argument("--pamp-l10", type=int, default=1,
                    help="single-wavefunction pAMP leg: hydrogen lmax 10, 150 B-splines, 20 vectors (0 = skip)")
    ap.add_argument("--learned", type=int, default=1,
                    help="learned-preconditioner leg at the L<=5, l<=10, 80-spline helium model (0 = skip)")
    ap.add_argument("--eager", action="store_true",
                    help="host-driven GMRES loops (same kernels, visible one by one to a profiler)")
    ap.add_argument("--ensemble", type=int, default=256, help="members of the batched leg (0 = skip)")
    ap.add_argument("--pulse", type=int, default=1,
                    help="whole-pulse leg against the reference run at equal error (0 = skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    from pyprop_gb300 import build_native
    if args.profile == "matvec_hbm":
        build_native.build()
        profile_large_matvec()
        return
    if args.profile == "two_electron":
        build_native.build()
        profile_two_electron()
        return
    if args.profile == "two_electron_large":
        build_native.build()
        profile_two_electron_large()
        return
    if args.profile == "pamp_l10":
        build_native.build()
        profile_pamp_l10()
        return
    if args.profile == "ensemble_pamp":
        build_native.build()
        profile_ensemble_pamp()
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        build_native.build()
        run_ours(args)


if __name__ == "__main__":
    main()
