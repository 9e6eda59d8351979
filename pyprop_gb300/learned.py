"""Learned preconditioner for the Cayley GMRES solve.

The reference's Cayley step is preconditioned by fixed factorizations (the block-diagonal
radial solve, ``pyprop/propagator/CayleyPropagator.py:56-63,91-96``); there is no learned
part. Here a small network corrects the block-diagonal preconditioner for the coupling it
leaves out:

    P(v) = y + s(t) * MLP(features(y)),    y = M^-1 v (block-diagonal radial LU)

with ``features`` the block and its two angular neighbours, ``s(t) = i dt/2 E(t)`` the
strength of the time-dependent coupling, and the network trained on residual/correction
pairs that the plain solver produces along a propagation (``LearnedPreconditioner.harvest``).
The network runs on the device (``pg_mlp_*``: BF16 weights, FP32 accumulation, forward,
backward and Adam in this package's kernels). Inside the Cayley step it preconditions
flexible GMRES, and the FP64 true residual judges every refinement pass: a pass that does
not halve the residual is discarded and the step continues with the block-diagonal solve
alone (the fallback).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat
from .gpu import Context, check, ptr


def features_width(N):
    """Network input width for radial size N: three complex blocks, padded to 16."""
    return ((6 * N + 15) // 16) * 16


class MlpNet:
    """Device MLP (``pg_mlp``): d_in -> hidden -> hidden -> d_out, bias-free, ReLU."""

    def __init__(self, d_in, hidden, d_out, seed=7, ctx=None):
        self.ctx = ctx or Context.get()
        self.lib = self.ctx.lib
        self.d_in, self.hidden, self.d_out = int(d_in), int(hidden), int(d_out)
        h = C.c_void_p()
        check(self.lib.pg_mlp_create(self.ctx.h, self.d_in, self.hidden, self.d_out, int(seed), C.byref(h)),
              "pg_mlp_create")
        self.h = h
        self.shapes = [(self.d_in, self.hidden), (self.hidden, self.hidden), (self.hidden, self.d_out)]

    def parameter_count(self):
        return int(self.lib.pg_mlp_parameter_count(self.h))

    def get_weights(self):
        flat = np.zeros(self.parameter_count(), dtype=np.float32)
        check(self.lib.pg_mlp_get_weights(self.h, flat.ctypes.data), "pg_mlp_get_weights")
        return self._split(flat)

    def set_weights(self, weights):
        flat = np.ascontiguousarray(np.concatenate([np.asarray(w, dtype=np.float32).ravel() for w in weights]))
        if flat.size != self.parameter_count():
            raise ValueError("weight count %d, expected %d" % (flat.size, self.parameter_count()))
        check(self.lib.pg_mlp_set_weights(self.h, flat.ctypes.data), "pg_mlp_set_weights")

    def _split(self, flat):
        out, o = [], 0
        for r, c in self.shapes:
            out.append(flat[o:o + r * c].reshape(r, c).copy())
            o += r * c
        return out

    def forward(self, X, Y):
        """Y (float32 [batch][d_out], device) = MLP(X (bfloat16 [batch][d_in], device))."""
        self.ctx.bind_stream()
        check(self.lib.pg_mlp_forward(self.h, ptr(X), X.shape[0], ptr(Y)), "pg_mlp_forward")

    def gradients(self, X, T):
        """(loss, [g1, g2, g3]) of mean_rows ||MLP(X) - T||^2 (host float32 gradients)."""
        self.ctx.bind_stream()
        loss = C.c_double(0.0)
        flat = np.zeros(self.parameter_count(), dtype=np.float32)
        check(self.lib.pg_mlp_gradients(self.h, ptr(X), ptr(T), X.shape[0], C.byref(loss), flat.ctypes.data),
              "pg_mlp_gradients")
        return loss.value, self._split(flat)

    def train_step(self, X, T, lr, want_loss=False):
        self.ctx.bind_stream()
        loss = C.c_double(0.0)
        check(self.lib.pg_mlp_train_step(self.h, ptr(X), ptr(T), X.shape[0], C.c_float(lr),
                                         C.byref(loss) if want_loss else None), "pg_mlp_train_step")
        return loss.value if want_loss else None

    def block_features(self, y, X):
        """X (bfloat16 [nblk][d_in]) = features of y (complex64 [nblk][N]), both on the device."""
        self.ctx.bind_stream()
        nblk, N = y.shape
        check(self.lib.pg_mlp_block_features(self.ctx.h, ptr(y), nblk, N, self.d_in, ptr(X)), "pg_mlp_block_features")

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.pg_mlp_destroy(self.h)
        except Exception:
            pass


class LearnedPreconditioner:
    """Network, training data and training for one CayleyPropagatorGPU (mixed precision).

    ``harvest(prob, nsteps)`` propagates with the plain solver and keeps, per step, the
    residual r = (S - i dt/2 H) psi_n - (S + i dt/2 H) psi_n of the starting guess psi_n and
    the converged correction e = psi_{n+1} - psi_n (A e = r). The network learns, per angular
    block a, t_a = (e_a - y_a) / (s |y|) from features(y / |y|), y = M^-1 r: the part of the
    exact correction that the block preconditioner misses, per unit coupling strength.
    """

    def __init__(self, prop, hidden=256, seed=7, coupling_potential=None):
        """coupling_potential: index (in the propagator's potential list) of the term whose
        scale i dt/2 h(t) multiplies the correction - by default the one time-dependent term
        (the field coupling the block preconditioner leaves out); a time-independent term gives
        the constant scale i dt/2 (for a part of H the preconditioner omits at all times, such
        as the two-electron repulsion)."""
        shape = prop.psi.GetRepresentation().GetFullShape()
        self.prop = prop
        self.shape = shape
        self.nblk, self.N = shape[0], int(np.prod(shape[1:]))  # one network row per angular channel
        self.d_in = features_width(self.N)
        self.d_out = ((2 * self.N + 7) // 8) * 8
        self.net = MlpNet(self.d_in, hidden, self.d_out, seed=seed, ctx=prop.op64.ctx)
        pots = prop.BasePropagator.PotentialList
        if coupling_potential is None:
            dep = [p for p, pot in enumerate(pots) if pot.IsTimeDependent]
            if len(dep) != 1:
                raise ValueError("give coupling_potential: the propagator has %d time-dependent terms" % len(dep))
            coupling_potential = dep[0]
        self.pot_index = int(coupling_potential)
        self.slot = 1 + self.pot_index  # slot of that potential in the device operator (slot 0: overlap)
        self.pairs = []

    def coupling_scale(self, t, dt):
        return 0.5j * dt * self.prop.BasePropagator.PotentialList[self.pot_index].GetTimeScaling(t + abs(dt) / 2.0)

    def harvest(self, prob, nsteps):
        import torch
        prop = self.prop
        dt = prob.TimeStep
        for _ in range(nsteps):
            t = prob.PropagatedTime
            psi = prob.psi.GetData()
            psi0 = psi.clone()
            r = torch.zeros_like(psi0)
            prop.op64.matvec(prop.op64.scales(t + abs(dt) / 2.0, -1j * dt, 0.0), psi0, r)
            prob.AdvanceStep()
            e = prob.psi.GetData() - psi0
            self.pairs.append((t, dt, r.to(torch.complex64), e.to(torch.complex64)))
        return len(self.pairs)

    def _block_solve(self, r):
        y = r.clone()
        self.prop.Preconditioner.solvers[nat.PG_FP32].apply(nat.PG_BAND_PREC_SOLVE, y)
        return y

    def training_set(self, pairs, rng=None, phases=1, min_field=1e-3):
        """(X bf16 [rows][d_in], T float32 [rows][d_out]) on the device; pairs whose coupling
        scale is below min_field times the largest are skipped (nothing to learn there)."""
        import torch
        smax = max(abs(self.coupling_scale(t, dt)) for t, dt, _, _ in pairs)
        Xs, Ts = [], []
        for t, dt, r, e in pairs:
            s = self.coupling_scale(t, dt)
            if abs(s) < min_field * smax:
                continue
            y = self._block_solve(r).reshape(self.nblk, self.N)
            e = e.reshape(self.nblk, self.N)
            ny = float(torch.linalg.vector_norm(y))
            for k in range(phases):
                ph = 1.0 if (rng is None or k == 0) else complex(np.exp(1j * rng.uniform(0, 2 * np.pi)))
                yk = (y * ph / ny).contiguous()
                X = torch.empty((self.nblk, self.d_in), dtype=torch.bfloat16, device=y.device)
                self.net.block_features(yk, X)
                tgt = ((e * ph - y * ph) / (s * ny)).contiguous()
                T = torch.zeros((self.nblk, self.d_out), dtype=torch.float32, device=y.device)
                T[:, :2 * self.N] = torch.view_as_real(tgt).reshape(self.nblk, 2 * self.N)
                Xs.append(X)
                Ts.append(T)
        return torch.cat(Xs), torch.cat(Ts)

    def train(self, X, T, steps=400, lr=1e-3, batch=1024, seed=0):
        import torch
        g = torch.Generator(device="cpu").manual_seed(seed)
        losses = []
        rows = X.shape[0]
        for k in range(steps):
            idx = torch.randint(0, rows, (min(batch, rows),), generator=g).to(X.device)
            want = (k % 50 == 0) or k == steps - 1
            loss = self.net.train_step(X[idx].contiguous(), T[idx].contiguous(), lr, want_loss=want)
            if want:
                losses.append(loss)
        return losses

    def apply(self, r, t, dt, learned=True):
        """P(r) (complex64 [nblk][N]) with or without the learned correction."""
        import torch
        y = self._block_solve(r)
        if not learned:
            return y
        yb = y.reshape(self.nblk, self.N).contiguous()
        X = torch.empty((self.nblk, self.d_in), dtype=torch.bfloat16, device=y.device)
        self.net.block_features(yb, X)
        out = torch.empty((self.nblk, self.d_out), dtype=torch.float32, device=y.device)
        self.net.forward(X, out)
        corr = torch.view_as_complex(out[:, :2 * self.N].reshape(self.nblk, self.N, 2).contiguous())
        return (yb + self.coupling_scale(t, dt) * corr).reshape(y.shape)

    def one_step_residual(self, pairs, learned=True):
        """Mean over pairs of ||A P(r) - r|| / ||r|| (A = S + i dt/2 H(t + dt/2), complex64)."""
        import torch
        op = self.prop.opb
        vals = []
        for t, dt, r, _ in pairs:
            z = self.apply(r, t, dt, learned).contiguous()
            Az = torch.zeros_like(z)
            op.matvec(op.scales(t + abs(dt) / 2.0, 0.5j * dt, 1.0), z, Az)
            vals.append(float(torch.linalg.vector_norm(Az - r) / torch.linalg.vector_norm(r)))
        return float(np.mean(vals))

    def attach(self, on=True):
        """Use (or stop using) the network inside the propagator's Cayley steps."""
        self.prop.stepper.set_learned(self.net if on else None, self.slot)

    def compare_steps(self, prob, nsteps):
        """nsteps Cayley steps from prob's current state without and with the network (each
        after one untimed step from the same state, which the timed run restarts from):
        {"block": ..., "learned": ...} with the GMRES iterations, the device time in ms, the
        largest FP64 true residual and the passes the judge rejected, and "relerr" between
        the two final states. prob ends in the learned run's final state, network detached."""
        import torch
        start = prob.psi.GetData().clone()
        t0 = prob.PropagatedTime
        out, psis = {}, {}
        for on in (False, True):
            self.attach(on)
            rej0 = self.prop.stepper.learned_rejected() if on else 0
            for timed in (False, True):
                prob.psi.GetData().copy_(start)
                prob.PropagatedTime = t0
                if not timed:
                    prob.AdvanceStep()
                    continue
                torch.cuda.synchronize()
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                it, res = 0, 0.0
                s.record()
                for _ in range(nsteps):
                    prob.AdvanceStep()
                    st = self.prop.LastStats
                    it += st.Iterations
                    res = max(res, st.TrueResidual)
                e.record()
                e.synchronize()
                out["learned" if on else "block"] = {
                    "gmres_iterations": int(it), "ms": s.elapsed_time(e), "max_true_residual": res,
                    "rejected_passes": (self.prop.stepper.learned_rejected() - rej0) if on else 0}
                psis[on] = prob.psi.GetData().clone()
        self.attach(False)
        out["relerr"] = float(torch.linalg.vector_norm(psis[True] - psis[False]) / torch.linalg.vector_norm(psis[False]))
        return out
