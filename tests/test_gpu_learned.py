"""Learned preconditioner network on the GPU vs the CPU oracle (gradient check, training)."""
import numpy as np
import pytest

from tests.helpers import relerr

pytestmark = pytest.mark.gpu


def _net(d_in, hidden, d_out, seed=3):
    from pyprop_gb300.learned import MlpNet
    return MlpNet(d_in, hidden, d_out, seed=seed)


def test_forward_and_gradients_match_oracle(gpu):
    import torch
    from oracle.mlp import bf16, forward, loss_and_gradients
    rng = np.random.default_rng(4)
    d_in, h, d_out, B = 96, 64, 48, 37
    net = _net(d_in, h, d_out)
    W = [rng.standard_normal((d_in, h)) * np.sqrt(2.0 / d_in), rng.standard_normal((h, h)) * np.sqrt(2.0 / h),
         rng.standard_normal((h, d_out)) * np.sqrt(1.0 / h)]
    net.set_weights(W)
    Wd = net.get_weights()
    assert max(np.abs(a - b).max() for a, b in zip(Wd, W)) < 1e-6
    X = bf16(rng.standard_normal((B, d_in)))
    T = rng.standard_normal((B, d_out))
    Xd = torch.as_tensor(X, dtype=torch.float32, device="cuda").to(torch.bfloat16)
    Td = torch.as_tensor(T, dtype=torch.float32, device="cuda")
    Y = torch.zeros((B, d_out), dtype=torch.float32, device="cuda")
    net.forward(Xd, Y)
    y_ref = forward(W, X)[2]
    assert relerr(Y.cpu().numpy(), y_ref) < 1e-2
    loss, g = net.gradients(Xd, Td)
    loss_ref, g_ref = loss_and_gradients(W, X, T)
    assert abs(loss - loss_ref) < 1e-3 * loss_ref
    for layer in range(3):
        assert relerr(g[layer], g_ref[layer]) < 2e-2, (layer, relerr(g[layer], g_ref[layer]))


def test_training_reduces_loss_on_a_linear_target(gpu):
    import torch
    rng = np.random.default_rng(5)
    d_in, h, d_out, B = 64, 256, 32, 512
    A = rng.standard_normal((d_in, d_out)) / np.sqrt(d_in)
    X = rng.standard_normal((B, d_in))
    T = X @ A
    net = _net(d_in, h, d_out, seed=11)
    Xd = torch.as_tensor(X, dtype=torch.float32, device="cuda").to(torch.bfloat16)
    Td = torch.as_tensor(T, dtype=torch.float32, device="cuda")
    # where a non-finite first loss would come from: the initial weights, the inputs, the output
    W0 = net.get_weights()
    Y0 = torch.zeros((B, d_out), dtype=torch.float32, device="cuda")
    net.forward(Xd, Y0)
    stages = {"weights": all(bool(np.isfinite(w).all()) for w in W0), "X": bool(torch.isfinite(Xd.float()).all()),
              "T": bool(torch.isfinite(Td).all()), "Y": bool(torch.isfinite(Y0).all())}
    first = net.train_step(Xd, Td, 1e-3, want_loss=True)
    assert np.isfinite(first), stages
    for _ in range(400):
        net.train_step(Xd, Td, 1e-3)
    last = net.train_step(Xd, Td, 1e-3, want_loss=True)
    assert last < 0.05 * first, (first, last)


def _strong_field_problem(precision="fp32"):
    from tests.helpers import hydrogen_problem
    return hydrogen_problem(lmax=7, nbsplines=40, rmax=40.0, propagator="CayleyPropagatorGPU", precision=precision,
                            gmres_tolerance=1e-12, amplitude=0.1, pulse_duration=4.0, duration=4.0)


def test_learned_cayley_steps_match_the_plain_path(gpu):
    """Flexible GMRES with the (untrained) learned preconditioner reaches the same states."""
    from pyprop_gb300.learned import LearnedPreconditioner
    from tests.helpers import golden
    plain = _strong_field_problem()
    plain.SetupStep(skipWavefunctionSetup=True)
    learned = _strong_field_problem()
    learned.SetupStep(skipWavefunctionSetup=True)
    lp = LearnedPreconditioner(learned.Propagator, hidden=64)
    lp.attach()
    rng = np.random.default_rng(0)
    psi = rng.standard_normal(plain.psi.GetData().shape) + 0j
    import torch
    for p in (plain, learned):
        p.psi.GetData().copy_(torch.as_tensor(psi / np.linalg.norm(psi), device="cuda"))
        p.PropagatedTime = 1.0
    for _ in range(10):
        plain.AdvanceStep()
        learned.AdvanceStep()
        assert learned.Propagator.LastStats.TrueResidual < 1e-12
    assert relerr(learned.psi.numpy(), plain.psi.numpy()) < 1e-10
    assert learned.Propagator.stepper.learned_rejected() == 0


def test_trained_network_improves_the_block_preconditioner(gpu):
    """Trained on the plain solver's residual/correction pairs, the learned correction lowers
    the one-step residual ||A P(r) - r|| / ||r|| on held-out steps, and the learned Cayley
    steps need no more GMRES iterations than the plain ones."""
    import torch
    from pyprop_gb300.learned import LearnedPreconditioner
    prob = _strong_field_problem()
    prob.SetupStep(skipWavefunctionSetup=True)
    psi = np.zeros(prob.psi.GetData().shape, dtype=np.complex128)
    rng = np.random.default_rng(1)
    psi[0] = rng.standard_normal(psi.shape[1])
    psi[1] = 0.3 * rng.standard_normal(psi.shape[1])
    prob.psi.GetData().copy_(torch.as_tensor(psi / np.linalg.norm(psi), device="cuda"))
    prob.PropagatedTime = 0.5
    lp = LearnedPreconditioner(prob.Propagator, hidden=256, seed=3)
    lp.harvest(prob, 160)
    train, held = lp.pairs[:120], lp.pairs[120:]
    X, T = lp.training_set(train, rng=np.random.default_rng(2), phases=4)
    losses = lp.train(X, T, steps=600, lr=1e-3, batch=512)
    assert losses[-1] < 0.5 * losses[0], losses
    plain_rho = lp.one_step_residual(held, learned=False)
    learned_rho = lp.one_step_residual(held, learned=True)
    print("one-step residual: block %.3e, learned %.3e; loss %.3e -> %.3e" % (plain_rho, learned_rho, losses[0],
                                                                            losses[-1]))
    assert learned_rho < plain_rho
    # in the Cayley step: continue the propagation with and without the network
    state = prob.psi.GetData().clone()
    t0 = prob.PropagatedTime
    iters = {}
    for use in (False, True):
        lp.attach(use)
        prob.psi.GetData().copy_(state)
        prob.PropagatedTime = t0
        n = 0
        for _ in range(20):
            prob.AdvanceStep()
            st = prob.Propagator.LastStats
            assert st.TrueResidual < 1e-12
            n += st.Iterations
        iters[use] = n
    print("GMRES iterations over 20 steps: block %d, learned %d" % (iters[False], iters[True]))
    assert iters[True] <= iters[False]


def test_learned_preconditioner_on_the_two_electron_model(gpu):
    """Helium in a laser field, Cayley steps preconditioned by the Kronecker radial block
    preconditioner (which leaves out the electron-electron repulsion): the network, trained on
    the solver's own residual/correction pairs with the repulsion's constant scale i dt/2,
    lowers the one-step residual on held-out steps; the learned Cayley steps reach the same
    states with the FP64 true residual below tolerance."""
    import torch
    from pyprop_gb300.learned import LearnedPreconditioner
    from tests.helpers import helium_problem
    prob = helium_problem(lmax=1, nbsplines=14, rmax=12.0, L=(0, 1), amplitude=0.1, frequency=1.0,
                          pulse_duration=4.0, duration=4.0, propagator="CayleyPropagatorGPU", precision="fp32",
                          preconditioner_type="TwoElectronKroneckerPreconditioner")
    prob.SetupStep(skipWavefunctionSetup=True)
    assert prob.Propagator.Preconditioner.__class__.__name__ == "TwoElectronKroneckerPreconditioner"
    pots = prob.Propagator.BasePropagator.PotentialList
    r12 = [i for i, p in enumerate(pots) if "ElectronicCoupling" in p.Name][0]
    shape = prob.psi.GetRepresentation().GetFullShape()
    rng = np.random.default_rng(10)
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    prob.psi.GetData().copy_(torch.as_tensor(psi / np.linalg.norm(psi), device="cuda"))
    prob.PropagatedTime = 0.5
    lp = LearnedPreconditioner(prob.Propagator, hidden=256, seed=5, coupling_potential=r12)
    lp.harvest(prob, 120)
    train, held = lp.pairs[:90], lp.pairs[90:]
    X, T = lp.training_set(train, rng=np.random.default_rng(3), phases=4)
    losses = lp.train(X, T, steps=600, lr=1e-3, batch=512)
    plain_rho = lp.one_step_residual(held, learned=False)
    learned_rho = lp.one_step_residual(held, learned=True)
    print("helium one-step residual: Kronecker block %.3e, learned %.3e; loss %.3e -> %.3e" % (
        plain_rho, learned_rho, losses[0], losses[-1]))
    assert losses[-1] < 0.5 * losses[0]
    assert learned_rho < plain_rho
    state = prob.psi.GetData().clone()
    t0 = prob.PropagatedTime
    out, iters = {}, {}
    for use in (False, True):
        lp.attach(use)
        prob.psi.GetData().copy_(state)
        prob.PropagatedTime = t0
        n = 0
        for _ in range(10):
            prob.AdvanceStep()
            st = prob.Propagator.LastStats
            assert st.TrueResidual < 1e-11
            n += st.Iterations
        iters[use], out[use] = n, prob.psi.numpy()
    print("helium GMRES iterations over 10 steps: block %d, learned %d" % (iters[False], iters[True]))
    # both meet the true-residual tolerance; their states agree to that tolerance times the
    # conditioning of S x S + i dt/2 H
    assert relerr(out[True], out[False]) < 1e-7
    assert iters[True] <= iters[False]


def test_learned_at_helium_l10_80_splines(gpu):
    """The learned preconditioner at the size it is specified on: helium, coupled L <= 5,
    l1, l2 <= 10, 80 B-splines per electron (291 angular blocks of 6400 coefficients), on top
    of the fast-diagonalization blocks, learning the repulsion they omit from 50 052 harvested
    block pairs. The network trains on the GPU (the loss falls), and the flexible steps with it
    meet the same true-residual tolerance and agree with the block-preconditioned steps to the
    GMRES tolerance. Its effect on the GMRES iterations is not asserted: at this size the
    network does not generalise to held-out residuals (its features are a channel and its two
    angular neighbours, while the repulsion couples every channel of the same L) and runs went
    from 120 to 115, 119 and 125 iterations over 20 steps; the counts are reported by the
    benchmark's learned leg."""
    import torch
    import bench
    out = bench.time_learned_helium(torch)
    assert out["pairs"] == 50052 and out["training_rows"] > 40000
    assert out["loss_last"] < out["loss_first"]
    assert out["block"]["max_true_residual"] < 1e-10 and out["learned"]["max_true_residual"] < 1e-10
    assert out["relerr"] < 1e-6
    assert out["learned"]["rejected_passes"] >= 0 and out["learned"]["gmres_iterations"] > 0
