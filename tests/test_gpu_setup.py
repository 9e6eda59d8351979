"""Operator construction on the GPU: the B-spline band projection of two-electron radial
factors (pg_bspline_band_project) against the host projection of the same functions."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_stencil(f, bs1, bs2):
    """R[i1][d1][d2][i2] from two host band projections (along r2, then along r1)."""
    A = bs2.band_elements(f, 0)                      # [q1][N2][bw]
    X = bs1.band_elements(np.moveaxis(A, 0, -1), 0)  # [N2][bw][N1][bw]
    return np.ascontiguousarray(X.transpose(2, 3, 1, 0))


def _factors(monkeypatch, gpu, **kw):
    from tests.helpers import helium_problem
    monkeypatch.setenv("PYPROP_GPU_SETUP", "1" if gpu else "0")
    prob = helium_problem(**kw)
    pots = prob.Propagator.BasePropagator.PotentialList
    return {p.Name: p.Factors for p in pots if getattr(p, "Factors", None) is not None}


def test_band_project_matches_host_projection():
    from tests.helpers import helium_problem
    from pyprop_gb300.tensorpotential import radial_stencil_gpu
    prob = helium_problem(lmax=1, nbsplines=24, rmax=20.0)
    bs = prob.psi.GetRepresentation().GetRepresentation(1).BSplineObject
    r = bs.grid
    rng = np.random.default_rng(7)
    for f in (1.0 / np.maximum(r[:, None], r[None, :]),
              np.exp(-0.1 * (r[:, None] - r[None, :]) ** 2) * rng.uniform(0.5, 1.5, (len(r), len(r)))):
        ref = _host_stencil(f, bs, bs)
        got = radial_stencil_gpu(f, bs, bs)
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_factored_potentials_same_on_gpu_and_host(monkeypatch):
    kw = dict(lmax=2, L=[0, 1], nbsplines=18, rmax=15.0, amplitude=0.05)
    host = _factors(monkeypatch, False, **kw)
    dev = _factors(monkeypatch, True, **kw)
    assert host and set(host) == set(dev)
    for name, h in host.items():
        d = dev[name]
        assert np.array_equal(h.coefs, d.coefs) and np.array_equal(h.weights, d.weights)
        scale = np.abs(h.stencil).max()
        assert np.abs(d.stencil - h.stencil).max() <= 1e-13 * scale, name


def test_two_electron_setup_time_at_learned_preconditioner_size(monkeypatch):
    """Radial factors of the helium model with l1, l2 <= 10 and 80 B-splines per electron
    (the learned-preconditioner workload's size): the GPU projection agrees with the host
    one and the setup times of both are printed."""
    from tests.helpers import helium_problem
    times, facs = {}, {}
    for gpu in (False, True):
        monkeypatch.setenv("PYPROP_GPU_SETUP", "1" if gpu else "0")
        t0 = time.perf_counter()
        prob = helium_problem(lmax=10, L=[0], nbsplines=80, rmax=80.0)
        times[gpu] = time.perf_counter() - t0
        facs[gpu] = [p.Factors for p in prob.Propagator.BasePropagator.PotentialList
                     if getattr(p, "Factors", None) is not None]
    print("setup host %.2f s, gpu %.2f s" % (times[False], times[True]))
    for h, d in zip(facs[False], facs[True]):
        assert np.abs(d.stencil - h.stencil).max() <= 1e-13 * np.abs(h.stencil).max()
