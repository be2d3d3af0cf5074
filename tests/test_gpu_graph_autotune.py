"""CUDA-graph capture and the launch-shape autotuner on the GPU.

Every launch shape runs the same per-mode arithmetic (only where the stage
vectors live and how many modes share an SM differ), and a captured graph
replays the same launches, so all comparisons here are bit for bit.
"""
import numpy as np
import pytest

import discoeb_gb300 as deb
import discoeb_gb300.background as bg
import discoeb_gb300.tables as tb
from discoeb_gb300 import _native, autotune
from discoeb_gb300 import perturbations as pt
from discoeb_gb300.gradient import GradientProblem, evolve_backgrounds, perturbed_params
from discoeb_gb300.workloads import sample_cosmologies

pytestmark = pytest.mark.gpu

FID = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17, nqmax=15)
SMALL = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)


@pytest.fixture(scope="module")
def two_cosmologies():
    params, _ = sample_cosmologies(2, seed=11)
    return params, [bg.evolve_background(param=p) for p in params]


def _problem(ps, dims, num_k=24):
    k = np.geomspace(1e-4, 10.0, num_k)
    tabs = tb.pack_batch(ps, dims["nqmax"])
    tau = np.stack([tb.tau_of_a(p, [1.0]) for p in ps])
    return deb.DeviceProblem(tabs, np.tile(k, len(ps)), tau, np.repeat(np.arange(len(ps), dtype=np.int32), num_k),
                             **dims)


def test_every_launch_shape_gives_identical_results(two_cosmologies):
    import torch

    _, ps = two_cosmologies
    prob = _problem(ps, FID)
    cfg = pt._cfg(1e-5, 1e-5, 0.25, 0.80, 0.0, 20.0, 0.3, 4096)
    ref = None
    seen = set()
    for cand in autotune.CANDIDATES:
        prob.plan = pt.get_plan(prob.dims, prob.nmode, cand)
        info = prob.plan.launch_info()
        seen.add(info["stage_vectors"])
        assert info["modes_in_flight"] >= 1
        prob.launch(cfg)
        torch.cuda.synchronize()
        assert (prob.status.cpu().numpy() == 0).all()
        y = prob.y.cpu().numpy().copy()
        if ref is None:
            ref = y
        else:
            np.testing.assert_array_equal(y, ref)
    assert seen == {"shared", "global", "all_global"}


def test_tune_keeps_the_fastest_measured_shape(two_cosmologies):
    _, ps = two_cosmologies
    prob = _problem(ps, FID, num_k=16)
    cfg = pt._cfg(1e-5, 1e-5, 0.25, 0.80, 0.0, 20.0, 0.3, 4096)
    times = prob.tune(cfg)
    assert len(times) >= 2 and all(t > 0 for t in times.values())
    info = prob.plan.launch_info()
    assert (info["stage_vectors"], info["modes_per_sm"]) == min(times, key=times.get)
    assert autotune.chosen(prob.dims) == min(times, key=times.get)


def test_forward_graph_replays_new_inputs_like_an_eager_launch(two_cosmologies):
    import torch

    _, ps = two_cosmologies
    prob = _problem([ps[0]], FID)
    cfg = pt._cfg(1e-5, 1e-5, 0.25, 0.80, 0.0, 20.0, 0.3, 4096)
    P0 = prob.capture(cfg, 4).clone()
    torch.cuda.synchronize()
    P1 = prob.replay().clone()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(P1.cpu().numpy(), P0.cpu().numpy())
    # new tables copied into the captured input buffer: the replay solves the new cosmology
    prob.tables.copy_(torch.as_tensor(tb.pack_batch([ps[1]], FID["nqmax"])))
    prob.tau_out.copy_(torch.as_tensor(np.stack([tb.tau_of_a(ps[1], [1.0])])))
    P2 = prob.replay().clone().cpu().numpy()
    fresh = _problem([ps[1]], FID)
    fresh.launch(cfg)
    P_ref = fresh.power(4).cpu().numpy()
    np.testing.assert_array_equal(P2, P_ref)
    assert not np.array_equal(P2, P0.cpu().numpy())


def test_gradient_graph_and_reloaded_inputs_match_eager_runs(two_cosmologies):
    import torch

    params, _ = two_cosmologies
    sets = []
    for p in params:
        pert = perturbed_params(p)
        flat = [p] + [q for (_, _, a, b) in pert for q in (a, b)]
        sets.append((p, pert, evolve_backgrounds(flat, processes=min(13, 4))))
    k = np.geomspace(1e-3, 1.0, 8)
    kw = dict(rtol=1e-5, atol=1e-5, max_steps=8000, **SMALL)
    (pa, perta, bga), (pb, pertb, bgb) = sets
    gp = GradientProblem([pa], [bga], [perta], k, [1.0], **kw)
    P0, D0 = (t.cpu().numpy().copy() for t in gp.run())
    gp.capture()
    P1, D1 = (t.cpu().numpy().copy() for t in gp.replay())
    np.testing.assert_array_equal(P1, P0)
    np.testing.assert_array_equal(D1, D0)
    gp.load([pb], [bgb], [pertb])
    P2, D2 = (t.cpu().numpy().copy() for t in gp.replay())
    gp.check()
    ref = GradientProblem([pb], [bgb], [pertb], k, [1.0], **kw)
    Pr, Dr = (t.cpu().numpy() for t in ref.run())
    np.testing.assert_array_equal(P2, Pr)
    np.testing.assert_array_equal(D2, Dr)
    torch.cuda.synchronize()


def test_public_gradient_call_reuses_its_graph(two_cosmologies):
    params, _ = two_cosmologies
    p = params[0]
    pert = perturbed_params(p)
    flat = [p] + [q for (_, _, a, b) in pert for q in (a, b)]
    bgs = evolve_backgrounds(flat, processes=4)
    kw = dict(aexp_out=[1.0], kmin=1e-3, kmax=1.0, num_k=8, rtol=1e-5, atol=1e-5, max_steps=8000, **SMALL)
    outs = [deb.evolve_perturbations_grad(params=p, backgrounds=[bgs], **kw) for _ in range(3)]
    for P, D, _ in outs[1:]:
        np.testing.assert_array_equal(P, outs[0][0])
        np.testing.assert_array_equal(D, outs[0][1])
    from discoeb_gb300 import gradient

    assert any(g.graph is not None for g in gradient._problems.values())
