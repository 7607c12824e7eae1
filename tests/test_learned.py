"""The learned proposal: CPU oracle pinned by finite differences, GPU kernels
against the oracle, and what the trained network gains in the search."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import mlp as om


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = om.init(1).astype(np.float64) + 0.01 * rng.standard_normal(om.N_PARAMS)
    x = rng.standard_normal((7, om.N_IN))
    y = rng.standard_normal((7, 2)) * 0.5
    _, g = om.loss_and_grad(p, x, y)
    for i in rng.choice(om.N_PARAMS, 40, replace=False):
        e = np.zeros(om.N_PARAMS)
        e[i] = 1e-6
        num = (om.loss_and_grad(p + e, x, y)[0] - om.loss_and_grad(p - e, x, y)[0]) / 2e-6
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, num, g[i])


def test_oracle_features_of_an_ar1_series():
    rng = np.random.default_rng(1)
    n, a = 20000, 0.6
    e = rng.standard_normal(n)
    y = np.zeros(n)
    for t in range(1, n):
        y[t] = a * y[t - 1] + e[t]
    f = om.features(y[None], [0, n])[0]
    np.testing.assert_allclose(f[:8], a ** np.arange(1, 9), atol=0.03)
    assert f[8] == n / 1000.0
    # no lag products across a run boundary
    z = np.ones((1, 10))
    f2 = om.features(z, [0, 5, 10])[0]
    assert f2[0] == pytest.approx(8 / 10)  # 4 + 4 lag-1 products over 10


def test_oracle_adam_step():
    p = np.ones(3)
    g = np.array([1.0, -2.0, 0.0])
    p1, m, v = om.adam(p, g, np.zeros(3), np.zeros(3), 1, lr=0.1)
    np.testing.assert_allclose(p1, [0.9, 1.1, 1.0], atol=1e-6)


# ------------------------------------------------------------------ GPU


@pytest.mark.gpu
def test_gpu_mlp_forward_grad_adam_match_oracle():
    from fastfuncstuff_gb300 import _lib
    from fastfuncstuff_gb300.glm import learned

    dev = torch.device("cuda:0")
    assert _lib.load().ffs_mlp_param_count() == om.N_PARAMS
    rng = np.random.default_rng(3)
    p = (om.init(5) + 0.02 * rng.standard_normal(om.N_PARAMS)).astype(np.float32)
    B = 1000
    x = rng.standard_normal((B, om.N_IN)).astype(np.float32)
    y = (rng.standard_normal((B, 2)) * 0.4).astype(np.float32)
    pt = torch.from_numpy(p).to(dev)
    xt, yt = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    out = learned.ArmaProposal(pt).forward(xt).cpu().numpy()
    np.testing.assert_allclose(out, om.forward(p, x), rtol=1e-4, atol=1e-5)
    grad = torch.zeros(om.N_PARAMS, device=dev)
    loss = torch.zeros(1, device=dev)
    learned.mlp_grad(pt, xt, yt, None, B, grad, loss)
    L, g = om.loss_and_grad(p.astype(np.float64), x, y)
    gg = grad.cpu().numpy()
    assert np.abs(gg - g).max() <= 1e-4 * np.abs(g).max(), np.abs(gg - g).max() / np.abs(g).max()
    assert float(loss.item()) == pytest.approx(L, rel=1e-4)
    # Adam consumes the gradient
    m = torch.zeros_like(grad)
    v = torch.zeros_like(grad)
    learned.adam(pt, grad, m, v, 1e-2, 1)
    p1, _, _ = om.adam(p.astype(np.float64), g, np.zeros_like(g), np.zeros_like(g), 1, lr=1e-2)
    np.testing.assert_allclose(pt.cpu().numpy(), p1, atol=2e-5)
    assert float(grad.abs().max()) == 0.0


@pytest.mark.gpu
def test_gpu_features_and_simulator():
    from fastfuncstuff_gb300 import synth
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    w = synth.workload(1, V=64)
    lay = G.run_layout(w.T, w.run_starts)
    X = torch.from_numpy(w.X).to(dev)
    V = 4000
    a = torch.full((V,), 0.6, device=dev)
    b = torch.full((V,), 0.2, device=dev)
    Y = learned.simulate(torch.zeros_like(X), lay, a, b, seed=11)  # zero design: sigma * noise
    yn = Y.cpu().numpy().astype(np.float64)
    var = yn.var(1, ddof=1)
    r1 = np.concatenate([(yn[:, 1:200] * yn[:, :199]).sum(1) / (199 * var),
                         (yn[:, 201:] * yn[:, 200:399]).sum(1) / (199 * var)]).mean()
    lam = (0.6 + 0.2) * (1 + 0.12) / (1 + 0.04 + 0.24)
    assert abs(r1 - lam) < 0.02, (r1, lam)
    # each run is standardised, then both share the voxel's sigma in U(0.5, 2)
    v1, v2 = yn[:, :200].var(1, ddof=1), yn[:, 200:].var(1, ddof=1)
    np.testing.assert_allclose(v1 / v2, 1.0, rtol=1e-4)
    assert 0.24 < v1.min() and v1.max() < 4.01
    # features of the residualised data against the oracle
    g = G.make_grid(torch.linspace(-0.8, 0.8, 9), torch.linspace(-0.8, 0.8, 9))
    f = engine.build_factors(X, g, lay, with_tc=False)
    Yd = torch.from_numpy(w.Y).to(dev)
    pre = engine.prep(Yd, f, tensor_core=False)
    feats = learned.features(Yd, f, lay).cpu().numpy()
    ref = om.features(pre.yr_t.t().cpu().numpy(), lay.run_start)
    np.testing.assert_allclose(feats, ref, rtol=1e-4, atol=1e-5)


@pytest.mark.gpu
def test_learned_search_agrees_with_full_grid_and_beats_untrained():
    """Train a small proposal on workload-1 designs, then compare the seeded
    search with the full-grid exhaustive argmin on held-out simulated voxels,
    and with the same search seeded by the untrained network."""
    from fastfuncstuff_gb300 import synth
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    w = synth.workload(1, V=64)
    lay = G.run_layout(w.T, w.run_starts)
    X = torch.from_numpy(w.X).to(dev)
    gr = torch.linspace(-0.8, 0.8, 33)
    f = engine.build_factors(X, G.make_grid(gr, gr), lay)
    x, y = learned.training_set(X, f, lay, 6_000_000, seed=5)  # the benchmark's training size
    prop, hist = learned.train(x, y, epochs=40, batch=8192, lr=3e-3, seed=1)
    # against the untrained network on the same held-out features
    out0 = learned.ArmaProposal(learned.init_params(1, dev)).forward(x[:50_000])
    loss0 = float(((out0 - y[:50_000]) ** 2).sum(1).mean().item() / 2)
    assert hist[-1]["holdout_loss"] < 0.2 * loss0
    # held-out voxels, (a, b) uniform over the valid grid
    a_t = torch.from_numpy(f.grid.a).to(dev)
    b_t = torch.from_numpy(f.grid.b).to(dev)
    idx = torch.randint(0, f.P, (50_000,), generator=torch.Generator().manual_seed(9)).to(dev)
    Y = learned.simulate(X, lay, a_t[idx], b_t[idx], seed=4242)
    full = engine.search(Y, f, hierarchical=False)
    seeded = learned.learned_search(Y, f, prop, lay, strip_k0=-1)  # the windows alone
    fb = seeded.fallback.float().mean().item()
    untrained = learned.learned_search(Y, f, learned.ArmaProposal(learned.init_params(1, dev)), lay, strip_k0=-1)
    fb0 = untrained.fallback.float().mean().item()
    assert fb < 0.8 * fb0  # the trained network keeps more voxels inside their window
    # the whole search (windows, one re-centred round, the strip next to the
    # identity line, full-grid fallback)
    rc = learned.learned_search(Y, f, prop, lay, recenter=1)
    agree_u = (rc.best == full.best).float().mean().item()
    # held-out voxels whose (a, b) follow the benchmark workload's
    # distribution: a ~ U(0.1, 0.8), b ~ U(-0.5, 0.3)
    gen = torch.Generator().manual_seed(11)
    a_w = (0.1 + 0.7 * torch.rand(100_000, generator=gen)).to(dev)
    b_w = (-0.5 + 0.8 * torch.rand(100_000, generator=gen)).to(dev)
    Yw = learned.simulate(X, lay, a_w, b_w, seed=777)
    full_w = engine.search(Yw, f, hierarchical=False)
    rw = learned.learned_search(Yw, f, prop, lay, recenter=1)
    same = rw.best == full_w.best
    agree = same.float().mean().item()
    gap = (rw.best_crit.double() - full_w.best_crit.double()) / full_w.best_crit.double().abs().clamp(min=1.0)
    print(f"learned: agreement {agree:.5f} (workload distribution), {agree_u:.5f} (uniform over the grid; "
          f"windows alone {(seeded.best == full.best).float().mean().item():.5f}); fallback {rw.stats['fallback']:.4f}, "
          f"strip voxels {int(rw.stats['strip_voxels'].item())}, gap of the disagreeing max "
          f"{float(gap[~same].max()) if bool((~same).any()) else 0.0:.2e}; untrained fallback {fb0:.4f}")
    assert agree >= 0.999
    assert agree_u >= 0.998
    # a voxel's answer is never below the global minimum (a window can only miss it)
    assert float(gap.min()) >= -1e-6
    # the strip only ever moves a voxel to the full grid
    assert float(rw.stats["fallback"]) >= 0.0


@pytest.mark.gpu
def test_strip_kernel_matches_full_grid_surface():
    """ffs_reml_strip sends to the full grid exactly the voxels whose least
    criterion over the strip next to the identity line (the full surface's
    values) lies below their window answer by more than 1e-6 of |crit0|,
    up to rounding next to that threshold, and only voxels of the device
    count compacted by ffs_reml_near_line."""
    from fastfuncstuff_gb300 import synth
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    w = synth.workload(1, V=3000)
    lay = G.run_layout(w.T, w.run_starts)
    X = torch.from_numpy(w.X).to(dev)
    gr = torch.linspace(-0.8, 0.8, 33)
    g = G.make_grid(gr, gr)
    f = engine.build_factors(X, g, lay)
    Y = torch.from_numpy(w.Y).to(dev)
    V = Y.shape[0]
    so = engine.search(Y, f, hierarchical=False, keep_surface=True)
    surf = so.surf.double().cpu().numpy()
    crit0 = so.crit0.cpu().numpy()
    n_b = len(g.b_axis)
    rng = np.random.default_rng(5)
    cells = rng.integers(0, len(g.a_axis) * n_b, V).astype(np.int32)  # windows anywhere
    out = dict(best=torch.empty(V, dtype=torch.int32, device=dev), dbest=torch.empty(V, device=dev),
               crit0=torch.empty(V, dtype=torch.float64, device=dev), fb=torch.zeros(V, dtype=torch.int32, device=dev),
               cell=torch.empty(V, dtype=torch.int32, device=dev))
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    pre = engine.prep(Y, f, want_yr_t=False, want_rows=True, split=False)
    learned._window_round(pre, f, torch.from_numpy(cells).to(dev), out, flag=flag)
    torch.cuda.synchronize()
    fb0 = out["fb"].cpu().numpy().copy()
    best = out["best"].cpu().numpy()
    dbest = out["dbest"].cpu().numpy().astype(np.float64)
    k0 = 6
    learned._strip_round(pre, f, out, flag=flag, k0=k0)
    torch.cuda.synchronize()
    assert int(flag.item()) == 0
    fb1 = out["fb"].cpu().numpy()
    cell1 = out["cell"].cpu().numpy()
    c = learned._window_consts(f)
    dist = c["dist_id"].cpu().numpy()
    strip = c["strip"]["pairs"].cpu().numpy()
    assert strip.size == 32 and (dist[strip] == 1).all()
    taken = (dist[best] <= k0) & (fb0 == 0)
    assert int(out["strip_voxels"].item()) == int(taken.sum())
    smin = surf[strip].min(0)
    thr = dbest - 1e-6 * np.abs(crit0)
    want = taken & (smin < thr)
    near = np.abs(smin - thr) <= 2e-7 * np.abs(crit0) + 1e-4  # rounding of the two kernels' sums
    assert want.any() and (taken & ~want).any()
    newly = (fb1 == 1) & (fb0 == 0)
    assert ((newly == want) | near).all()
    assert (cell1[newly] == -1).all()
    assert (fb1[fb0 == 1] == 1).all() and not newly[~taken].any()


@pytest.mark.gpu
def test_window_round_matches_full_grid_surface():
    """The 5 x 5 windows evaluated through the work-list tensor-core projection
    and the window kernel give the window argmin of the full surface
    (ffs_reml_surface, exhaustive), with (first identity pair, 0) as a
    candidate, the same criterion to the parity bar, and the edge flag of the
    window rule."""
    from fastfuncstuff_gb300 import synth
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    w = synth.workload(1, V=3000)
    lay = G.run_layout(w.T, w.run_starts)
    X = torch.from_numpy(w.X).to(dev)
    gr = torch.linspace(-0.8, 0.8, 33)
    g = G.make_grid(gr, gr)
    f = engine.build_factors(X, g, lay)
    Y = torch.from_numpy(w.Y).to(dev)
    V = Y.shape[0]
    so = engine.search(Y, f, hierarchical=False, keep_surface=True)
    surf = so.surf.double().cpu().numpy()
    crit0 = so.crit0.cpu().numpy()
    n_a, n_b = len(g.a_axis), len(g.b_axis)
    rng = np.random.default_rng(3)
    cells = rng.integers(0, n_a * n_b, V).astype(np.int32)
    # half of the voxels centred on their own full-grid argmin
    bi = so.best.cpu().numpy()
    for v in range(0, V, 2):
        p = bi[v]
        ai = np.searchsorted(g.a_axis, g.a[p])
        bj = np.searchsorted(g.b_axis, g.b[p])
        cells[v] = ai * n_b + bj
    out = dict(best=torch.empty(V, dtype=torch.int32, device=dev), dbest=torch.empty(V, device=dev),
               crit0=torch.empty(V, dtype=torch.float64, device=dev), fb=torch.zeros(V, dtype=torch.int32, device=dev),
               cell=torch.empty(V, dtype=torch.int32, device=dev))
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    pre = engine.prep(Y, f, want_yr_t=False, want_rows=True)
    counts = learned._window_round(pre, f, torch.from_numpy(cells).to(dev), out, flag=flag)
    torch.cuda.synchronize()
    assert int(flag.item()) == 0 and int(counts[1].item()) == 0
    ident = G.lambda_is_zero(g.a, g.b)
    p_id = int(np.nonzero(ident)[0][0])
    best = out["best"].cpu().numpy()
    dbest = out["dbest"].cpu().numpy()
    fb = out["fb"].cpu().numpy()
    np.testing.assert_allclose(out["crit0"].cpu().numpy(), crit0, rtol=1e-7)
    agree = 0
    for v in range(V):
        c = cells[v]
        ca, cb = divmod(int(c), n_b)
        a0 = min(max(ca - 2, 0), n_a - 5)
        b0 = min(max(cb - 2, 0), n_b - 5)
        cand, has_ident = [], False
        for ra in range(a0, a0 + 5):
            for rb in range(b0, b0 + 5):
                p = g.lattice[ra, rb]
                if p >= 0 and ident[p]:
                    has_ident = True
                if p >= 0 and not ident[p]:
                    cand.append((surf[p, v], int(p)))
        if not cand and not has_ident:  # no valid pair in the window: the full grid decides
            assert fb[v] == 1, v
            agree += 1
            continue
        d_ref, p_ref = min(cand) if cand else (np.inf, -1)
        if has_ident and (0.0, p_id) < (d_ref, p_ref if p_ref >= 0 else 1 << 30):
            d_ref, p_ref, exp_fb = 0.0, p_id, 0
        elif p_ref < 0 or d_ref >= 0:
            exp_fb = 1
        else:
            exp_fb = None  # the edge rule, below
        if best[v] == p_ref:
            agree += 1
        if p_ref < 0:
            continue
        # same criterion to the parity bar (crit = crit0 + d, 1e-6 relative)
        d_got_on_surface = 0.0 if ident[best[v]] else surf[best[v], v]
        scale_c = max(abs(crit0[v] + d_ref), 1.0)
        assert abs(d_got_on_surface - d_ref) <= 1e-6 * scale_c, (v, best[v], p_ref)
        assert abs(dbest[v] - d_got_on_surface) <= 1e-6 * scale_c, (v, dbest[v], d_got_on_surface)
        # edge rule
        if exp_fb is None:
            exp_fb = 0
            ba, bb = np.searchsorted(g.a_axis, g.a[p_ref]), np.searchsorted(g.b_axis, g.b[p_ref])
            for da in (-1, 0, 1):
                for db in (-1, 0, 1):
                    na, nb = ba + da, bb + db
                    if (da or db) and 0 <= na < n_a and 0 <= nb < n_b:
                        inside = a0 <= na < a0 + 5 and b0 <= nb < b0 + 5
                        if not inside and g.lattice[na, nb] >= 0:
                            exp_fb = 1
        if best[v] == p_ref:
            assert fb[v] == exp_fb, v
    assert agree / V >= 0.999, agree / V


@pytest.mark.gpu
@pytest.mark.parametrize("cuda_graphs", [True, False])
def test_fit_with_proposal_matches_full_grid_fit_where_pairs_agree(cuda_graphs):
    """fit_glm_arma11(proposal=...) queues the GLS of every voxel at its window
    pair, then redoes the fallback voxels at their full-grid pair: wherever the
    pair agrees with the full-grid fit the GLS outputs are identical (same
    kernels, same inputs), fallback voxels included. With CUDA graphs the
    fallback voxels' search and GLS replay from a graph of a padded voxel
    count beside the GLS graph; without, they run eagerly."""
    from fastfuncstuff_gb300 import fit_glm_arma11, synth
    from fastfuncstuff_gb300.glm import learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    w = synth.workload(1, V=6000)
    lay = G.run_layout(w.T, w.run_starts)
    X = torch.from_numpy(w.X).to(dev)
    Y = torch.from_numpy(w.Y).to(dev)
    gr = torch.linspace(-0.8, 0.8, 33)
    prop, _ = learned.train_proposal(X, lay, gr, gr, n_voxels=300_000, epochs=6)
    kw = dict(tr=2.0, a_grid=gr, b_grid=gr, run_starts=w.run_starts, device=dev, verbose=False,
              force_exhaustive_search=True, return_device=True, want_residuals=True)
    full = fit_glm_arma11(Y, X, **kw)
    got = fit_glm_arma11(Y, X, proposal=prop, proposal_recenter=1, cuda_graphs=cuda_graphs, **kw)
    again = fit_glm_arma11(Y, X, proposal=prop, proposal_recenter=1, cuda_graphs=cuda_graphs, **kw)
    assert torch.equal(got.betas, again.betas)  # a replay gives the same results
    # pinned host data: with graphs the prep streams the rows in place
    host = fit_glm_arma11(Y.cpu().pin_memory(), X, proposal=prop, proposal_recenter=1, cuda_graphs=cuda_graphs,
                          **kw)
    for name in ("betas", "tstats", "sigma2", "arma_params", "reml_likelihood", "residuals"):
        assert torch.equal(getattr(host, name), getattr(got, name)), name
    # results on the host (with graphs the GLS kernels write them into pinned
    # memory as they run, and the fallback voxels' rows are merged there)
    hout = fit_glm_arma11(Y.cpu().pin_memory(), X, proposal=prop, proposal_recenter=1, cuda_graphs=cuda_graphs,
                          **dict(kw, return_device=False))
    for name in ("betas", "tstats", "sigma2", "fstats", "r2", "arma_lambda", "arma_params", "reml_likelihood",
                 "residuals", "residuals_whitened"):
        assert not getattr(hout, name).is_cuda, name
        assert torch.equal(getattr(hout, name), getattr(got, name).cpu()), name
    same = (got.arma_params == full.arma_params).all(1)
    assert float(same.float().mean()) >= 0.995  # a briefly trained network
    assert 0.0 < float(got.learned_fallback) < 0.5  # some voxels took the fallback path
    for name in ("betas", "tstats", "sigma2", "fstats", "r2", "arma_lambda", "residuals", "residuals_whitened"):
        a, b = getattr(got, name)[same], getattr(full, name)[same]
        assert torch.equal(a, b), name


@pytest.mark.gpu
def test_proposal_trained_on_a_design_family_serves_a_held_out_design():
    """A proposal trained on a family of four workload-1-like designs (fresh
    task onsets and motion) serves a fifth design it never saw: on held-out
    voxels of that design the whole search agrees with the exhaustive full
    grid on >= 99.9% of voxels, and it sends at most a little more to the
    full-grid fallback than a proposal trained on the held-out design itself."""
    from fastfuncstuff_gb300 import synth
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    gr = torch.linspace(-0.8, 0.8, 33)
    lay = G.run_layout(400, [0, 200])
    family = torch.from_numpy(np.stack([synth.workload1_design(s) for s in (101, 102, 103, 104)])).to(dev)
    held = torch.from_numpy(synth.workload1_design(200)).to(dev)
    prop_fam, info = learned.train_proposal(family, lay, gr, gr)
    assert info["train_designs"] == 4
    prop_own, _ = learned.train_proposal(held, lay, gr, gr)
    f = engine.build_factors(held, G.make_grid(gr, gr), lay)
    gen = torch.Generator().manual_seed(21)
    a_w = (0.1 + 0.7 * torch.rand(100_000, generator=gen)).to(dev)
    b_w = (-0.5 + 0.8 * torch.rand(100_000, generator=gen)).to(dev)
    Y = learned.simulate(held, lay, a_w, b_w, seed=31)
    full = engine.search(Y, f, hierarchical=False)
    res = {}
    for name, prop in (("family", prop_fam), ("own", prop_own)):
        lo = learned.learned_search(Y, f, prop, lay, recenter=1)
        res[name] = ((lo.best == full.best).float().mean().item(), lo.stats["fallback"])
    print(f"held-out design: family-trained agreement {res['family'][0]:.5f}, fallback {res['family'][1]:.4f}; "
          f"own-design agreement {res['own'][0]:.5f}, fallback {res['own'][1]:.4f}")
    assert res["family"][0] >= 0.999
    assert res["family"][1] <= 1.5 * res["own"][1] + 0.005


@pytest.mark.gpu
@pytest.mark.parametrize("cuda_graphs", [True, False])
def test_learned_fit_with_t_not_a_multiple_of_four(cuda_graphs):
    """T = 398 (two runs of 199): the learned path needs no 16-byte rows (the
    window, strip and gather kernels take their per-sample paths, the graph
    copies the data into its buffer instead of reading it in place); where the
    pair agrees with the full-grid fit the GLS outputs are identical."""
    from fastfuncstuff_gb300 import fit_glm_arma11, synth
    from fastfuncstuff_gb300.glm import learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    w = synth.workload(1, V=5000)
    keep = np.ones(400, bool)
    keep[[199, 399]] = False
    Yn, Xn = np.ascontiguousarray(w.Y[:, keep]), np.ascontiguousarray(w.X[keep])
    lay = G.run_layout(398, [0, 199])
    X = torch.from_numpy(Xn).to(dev)
    Y = torch.from_numpy(Yn).to(dev)
    gr = torch.linspace(-0.8, 0.8, 33)
    prop, _ = learned.train_proposal(X, lay, gr, gr, n_voxels=300_000, epochs=6)
    kw = dict(tr=2.0, a_grid=gr, b_grid=gr, run_starts=[0, 199], device=dev, verbose=False,
              force_exhaustive_search=True, return_device=True)
    full = fit_glm_arma11(Y, X, **kw)
    got = fit_glm_arma11(Y, X, proposal=prop, proposal_recenter=1, cuda_graphs=cuda_graphs, **kw)
    host = fit_glm_arma11(Y.cpu().pin_memory(), X, proposal=prop, proposal_recenter=1, cuda_graphs=cuda_graphs,
                          **kw)
    assert torch.equal(host.betas, got.betas)
    same = (got.arma_params == full.arma_params).all(1)
    assert float(same.float().mean()) >= 0.99
    for name in ("betas", "tstats", "sigma2", "r2"):
        assert torch.equal(getattr(got, name)[same], getattr(full, name)[same]), name


@pytest.mark.gpu
def test_grouped_learned_fit_equals_per_group_learned_fits():
    """fit_glm_arma11_grouped with a proposal: one grid build over every
    design, the voxels in the grouped search's design slots, window rounds
    whose rows are sorted by design and window centre (every work item and
    criterion tile of one design). Each voxel's arithmetic is that of the
    learned search of its group alone against that design's view of the
    build, the strip next to the identity line included: the same pairs and
    GLS outputs bit for bit (workload-2 shapes: 4
    censored runs, N=855, 6 of the 20 designs); the pairs agree with the
    grouped exhaustive full grid where the windows hold the answer."""
    from fastfuncstuff_gb300 import fit_glm_arma11_grouped, synth
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    dev = torch.device("cuda:0")
    w = synth.workload(2, V=4000)
    keep = np.isin(w.groups, np.arange(6))
    Y, gid = w.Y[keep], w.groups[keep]
    designs = {h: w.designs[h] for h in range(6)}
    gr = torch.linspace(-0.8, 0.8, 33)
    lay = G.run_layout(w.Y.shape[1], w.run_starts, w.tau)
    fam = torch.stack([torch.from_numpy(designs[h]) for h in range(6)]).to(dev)
    prop, _ = learned.train_proposal(fam, lay, gr, gr, n_voxels=300_000, epochs=6)
    kw = dict(a_grid=gr, b_grid=gr, run_starts=w.run_starts, tau=w.tau, device=dev, verbose=False,
              force_exhaustive_search=True, want_residuals=True)
    got = fit_glm_arma11_grouped(Y, designs, gid, tr=2.0, proposal=prop, proposal_recenter=1, **kw)
    assert 0.0 <= float(got.learned_fallback) < 0.5
    grid = G.make_grid(gr, gr)
    f_all = engine.build_factors(fam, grid, lay)
    for h in range(6):
        m = gid == h
        Yh = torch.from_numpy(Y[m]).to(dev)
        fv = engine.design_view(f_all, h, center_flag=engine.constant_flag(fam[h])[0])
        lo = learned.learned_search(Yh, fv, prop, lay, recenter=1)
        go = engine.gls(Yh, lo.scale, lo.best, fv, fam[h], want_residuals=True)
        best = lo.best.cpu().numpy()
        np.testing.assert_array_equal(got.arma_params.numpy()[m], np.stack([grid.a[best], grid.b[best]], 1))
        np.testing.assert_array_equal(got.reml_likelihood.numpy()[m], lo.best_crit.cpu().numpy())
        for name, ref in (("betas", go.betas), ("tstats", go.tstats), ("sigma2", go.sigma2), ("r2", go.r2),
                          ("residuals", go.resid), ("residuals_whitened", go.resid_w)):
            np.testing.assert_array_equal(getattr(got, name).numpy()[m], ref.cpu().numpy(), err_msg=name)
    full = fit_glm_arma11_grouped(Y, designs, gid, tr=2.0, **kw)
    same = (got.arma_params == full.arma_params).all(1)
    assert float(same.float().mean()) >= 0.97
    np.testing.assert_array_equal(got.betas.numpy()[same.numpy()], full.betas.numpy()[same.numpy()])
