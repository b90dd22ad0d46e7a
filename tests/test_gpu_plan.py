"""Plans (geometry reused across density vectors) and batches (many plans in
one CUDA-graph launch) against the driver entries.

A plan evaluated for nv density vectors must give, vector by vector, what the
driver gives for that vector with the plan's parameters (FP64 form: to 1e-12
relative); a batch must give what its plans give one by one, whether the
captured graph is replayed or the work is launched eagerly.
"""
import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def _ft():
    import fasttools2d_gb300 as ft

    return ft


def _geom(seed, n, Lx, Ly, ntar=None):
    rng = np.random.default_rng(seed)
    ntar = n if ntar is None else ntar
    xs, ys = (rng.random(n) - 0.5) * Lx, (rng.random(n) - 0.5) * Ly
    xt, yt = (rng.random(ntar) - 0.5) * Lx, (rng.random(ntar) - 0.5) * Ly
    th = rng.random(n) * 2 * np.pi
    return xs, ys, xt, yt, np.cos(th), np.sin(th)


def _dens(seed, nv, n):
    rng = np.random.default_rng(seed)
    f1, f2 = rng.standard_normal((nv, n)), rng.standard_normal((nv, n))
    return f1 - f1.mean(1, keepdims=True), f2 - f2.mean(1, keepdims=True)


def _driver(ft, kind, g, f1, f2, Lx, Ly, prm, ctx):
    xs, ys, xt, yt, n1, n2 = g
    kw = dict(P=prm.P, xi=prm.xi, Mx=prm.Mx, My=prm.My, nside_x=prm.nside_x, nside_y=prm.nside_y, ctx=ctx,
              parts=False)
    if kind == ft.KIND_SLP:
        out = ft.StokesSLP_ewald_2p(xs, ys, xt, yt, f1, f2, Lx, Ly, **kw)
    else:
        out = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, f1, f2, Lx, Ly, **kw)
    return np.asarray(out[0]), np.asarray(out[1])


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("nv", [1, 3, 4])
def test_plan_matches_driver(gpu_ctx, kind, nv):
    ft = _ft()
    Lx, Ly = 2.0, 1.0
    g = _geom(100 + kind, 6000, Lx, Ly, ntar=4500)
    f1s, f2s = _dens(200 + nv, nv, 6000)
    plan = ft.Plan(kind, g[0], g[1], g[2], g[3], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=1e-12, nvmax=4,
                   ctx=gpu_ctx)
    prm = plan.params
    u1, u2 = plan.execute(f1s, f2s)
    assert u1.shape == (nv, 4500)
    for v in range(nv):
        d1, d2 = _driver(ft, kind, g, f1s[v], f2s[v], Lx, Ly, prm, gpu_ctx)
        err = rel_max(np.stack([u1[v], u2[v]]), np.stack([d1, d2]))
        assert err <= TOL_FP64, (kind, nv, v, err)
    # a second execute repeats the first up to the order of the atomic adds
    # that merge overlapping spread tiles into the grid
    w1, w2 = plan.execute(f1s, f2s)
    assert rel_max(np.stack([w1, w2]), np.stack([u1, u2])) <= 1e-14
    plan.close()


def test_plan_params_equal_driver_choice(gpu_ctx):
    """Created from the same density the plan chooses the driver's parameters."""
    ft = _ft()
    Lx, Ly = 1.0, 1.0
    g = _geom(7, 5000, Lx, Ly)
    f1s, f2s = _dens(8, 1, 5000)
    plan = ft.Plan(ft.KIND_SLP, g[0], g[1], g[2], g[3], f1s[0], f2s[0], Lx, Ly, tol=1e-10, ctx=gpu_ctx)
    u1, u2 = plan.execute(f1s, f2s)
    out, info = ft.StokesSLP_ewald_2p(g[0], g[1], g[2], g[3], f1s[0], f2s[0], Lx, Ly, tol=1e-10, ctx=gpu_ctx,
                                      return_info=True)
    p, q = plan.params, info.params
    assert (p.P, p.Mx, p.My, p.nside_x, p.nside_y) == (q.P, q.Mx, q.My, q.nside_x, q.nside_y)
    assert p.xi == q.xi
    assert rel_max(np.stack([u1[0], u2[0]]), np.stack([out[0], out[1]])) <= TOL_FP64


def test_plan_mixed_form(gpu_ctx):
    """A mixed-form plan meets its tolerance against the FP64 driver."""
    ft = _ft()
    Lx, Ly = 1.0, 1.0
    tol = 1e-8
    g = _geom(11, 20000, Lx, Ly)
    f1s, f2s = _dens(12, 3, 20000)
    for kind in (ft.KIND_SLP, ft.KIND_DLP):
        plan = ft.Plan(kind, g[0], g[1], g[2], g[3], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=tol,
                       form=ft.FORM_MIXED, ctx=gpu_ctx)
        u1, u2 = plan.execute(f1s, f2s)
        for v in range(3):
            xs, ys, xt, yt, n1, n2 = g
            if kind == ft.KIND_SLP:
                ref = ft.StokesSLP_ewald_2p(xs, ys, xt, yt, f1s[v], f2s[v], Lx, Ly, tol=1e-13, ctx=gpu_ctx,
                                            parts=False)
            else:
                ref = ft.StokesDLP_ewald_2p(xs, ys, xt, yt, n1, n2, f1s[v], f2s[v], Lx, Ly, tol=1e-13, ctx=gpu_ctx,
                                            parts=False)
            err = rel_max(np.stack([u1[v], u2[v]]), np.stack([ref[0], ref[1]]))
            assert err <= tol, (kind, v, err)
        plan.close()


def test_plan_device_tensors(gpu_ctx):
    torch = pytest.importorskip("torch")
    ft = _ft()
    Lx, Ly = 1.0, 1.5
    g = _geom(21, 3000, Lx, Ly)
    f1s, f2s = _dens(22, 2, 3000)
    T = [torch.tensor(a, device="cuda") for a in g]
    plan = ft.Plan(ft.KIND_DLP, T[0], T[1], T[2], T[3], torch.tensor(f1s[0], device="cuda"),
                   torch.tensor(f2s[0], device="cuda"), Lx, Ly, n1=T[4], n2=T[5], tol=1e-12, ctx=gpu_ctx)
    u1, u2 = plan.execute(torch.tensor(f1s, device="cuda"), torch.tensor(f2s, device="cuda"))
    torch.cuda.synchronize()
    plan_h = ft.Plan(ft.KIND_DLP, *g[:4], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=1e-12, ctx=gpu_ctx)
    h1, h2 = plan_h.execute(f1s, f2s)
    assert rel_max(np.stack([u1.cpu().numpy(), u2.cpu().numpy()]), np.stack([h1, h2])) <= TOL_FP64


def test_plan_rejects_too_many_vectors(gpu_ctx):
    ft = _ft()
    g = _geom(31, 500, 1.0, 1.0)
    f1s, f2s = _dens(32, 3, 500)
    plan = ft.Plan(ft.KIND_SLP, *g[:4], f1s[0], f2s[0], 1.0, 1.0, tol=1e-10, nvmax=2, ctx=gpu_ctx)
    with pytest.raises(ft.FteError):
        plan.execute(f1s, f2s)


def _batch_plans(ft, ctx, nv, form=0, tol=1e-10):
    rng = np.random.default_rng(41)
    plans, geoms, dens = [], [], []
    for i in range(7):
        n = int(np.exp(rng.uniform(np.log(800), np.log(20000))))
        Lx, Ly = [(1.0, 1.0), (2.0, 1.0), (1.0, 0.5), (1.5, 1.0)][i % 4]
        kind = i % 2
        g = _geom(300 + i, n, Lx, Ly)
        f1s, f2s = _dens(400 + i, nv, n)
        plans.append(ft.Plan(kind, *g[:4], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=tol, form=form, nvmax=nv,
                             ctx=ctx))
        geoms.append(g)
        dens.append((f1s, f2s))
    return plans, geoms, dens


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_plans(gpu_ctx, use_graph):
    ft = _ft()
    nv = 2
    plans, _, dens = _batch_plans(ft, gpu_ctx, nv)
    batch = ft.Batch(plans, nv, ctx=gpu_ctx)
    for i, (f1s, f2s) in enumerate(dens):
        batch.set_density(i, f1s, f2s)
    for rep in range(2):
        batch.launch(use_graph)
        for i, p in enumerate(plans):
            b1, b2 = batch.velocity(i)
            e1, e2 = p.execute(*dens[i])
            err = rel_max(np.stack([b1, b2]), np.stack([e1, e2]))
            assert err <= TOL_FP64, (rep, i, err)
    batch.close()


def test_batch_new_density_between_launches(gpu_ctx):
    """Replaying the graph after new densities are copied in uses the new data
    (an iterative solver's step)."""
    ft = _ft()
    nv = 1
    plans, _, dens = _batch_plans(ft, gpu_ctx, nv, form=ft.FORM_MIXED, tol=1e-8)
    batch = ft.Batch(plans, nv, ctx=gpu_ctx)
    for step in range(3):
        for i, p in enumerate(plans):
            f1s, f2s = _dens(1000 * step + i, nv, p.nsrc)
            dens[i] = (f1s, f2s)
            batch.set_density(i, f1s, f2s)
        batch.launch(True)
        for i, p in enumerate(plans):
            b1, b2 = batch.velocity(i)
            e1, e2 = p.execute(*dens[i])
            assert rel_max(np.stack([b1, b2]), np.stack([e1, e2])) <= 1e-12, (step, i)
    batch.close()


@pytest.mark.parametrize("form,tol", [(0, 1e-12), (1, 1e-6)])
def test_tuned_tiles_give_same_result(gpu_ctx, form, tol):
    """Tile sizes chosen by the autotuner change the work decomposition only:
    results agree with the default tiles (FP64 form to 1e-12; FP32 k-space
    within its tolerance) and the chosen sizes are reported."""
    ft = _ft()
    Lx, Ly = 1.5, 1.0
    g = _geom(51, 30000, Lx, Ly)
    f1s, f2s = _dens(52, 2, 30000)
    for kind in (ft.KIND_SLP, ft.KIND_DLP):
        base = ft.Plan(kind, *g[:4], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=tol, form=form, nvmax=2,
                       ctx=gpu_ctx)
        tuned = ft.Plan(kind, *g[:4], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=tol, form=form, nvmax=2,
                        tune=True, ctx=gpu_ctx)
        pb, pt = base.params, tuned.params
        assert (pb.Mx, pb.My, pb.P, pb.form) == (pt.Mx, pt.My, pt.P, pt.form)
        assert pt.ts_spread in (8, 12, 16, 20, 24, 32, 40, 48, 56, 64)
        assert pt.ts_gather in (8, 12, 16, 20, 24, 32, 40, 48, 56, 64)
        assert pb.ts_spread > 0 and pb.ts_gather > 0
        b1, b2 = base.execute(f1s, f2s)
        t1, t2 = tuned.execute(f1s, f2s)
        bar = 1e-12 if pb.form == ft.FORM_PLAIN else tol
        assert rel_max(np.stack([t1, t2]), np.stack([b1, b2])) <= bar, (kind, pt.ts_spread, pt.ts_gather)


def test_batch_work_lists_match_plans_in_few_launches(gpu_ctx):
    """A batch of mixed-form plans (float-float k-space: every stage one
    launch over all (plan, vector) items, the densities, zero modes and
    combinations one launch over all plans) gives, plan by plan and vector by
    vector, what the plans give one by one, in at most 100 kernel launches
    per step however many plans it holds; a plain (FP64) plan in the same
    batch takes the per-call path beside them."""
    ft = _ft()
    nv = 4
    rng = np.random.default_rng(77)
    plans, dens = [], []
    for i in range(24):
        n = int(np.exp(rng.uniform(np.log(1500), np.log(40000))))
        Lx, Ly = [(1.0, 1.0), (2.0, 1.0), (1.0, 0.75), (1.0, np.sqrt(2.0))][i % 4]
        g = _geom(900 + i, n, Lx, Ly)
        f1s, f2s = _dens(950 + i, nv, n)
        form, tol = (ft.FORM_PLAIN, 1e-10) if i == 5 else (ft.FORM_MIXED, 1e-8)
        plans.append(ft.Plan(i % 2, *g[:4], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=tol, form=form,
                             nvmax=nv, ctx=gpu_ctx))
        dens.append((f1s, f2s))
    assert sum(p.params.form == ft.FORM_FF for p in plans) >= 20
    batch = ft.Batch(plans, nv, ctx=gpu_ctx)
    for i, (f1s, f2s) in enumerate(dens):
        batch.set_density(i, f1s, f2s)
    k0 = gpu_ctx.kernel_count
    batch.launch(False)
    launches = gpu_ctx.kernel_count - k0
    # the plain plan alone launches ~10 kernels per vector on the per-call path
    assert launches <= 100, launches
    for use_graph in (True, False):
        batch.launch(use_graph)
        for i, p in enumerate(plans):
            b1, b2 = batch.velocity(i)
            e1, e2 = p.execute(*dens[i])
            assert rel_max(np.stack([b1, b2]), np.stack([e1, e2])) <= 1e-12, (use_graph, i, p.params.form)
    batch.close()
    for p in plans:
        p.close()


def test_batch_pinned_async_copies_match_synchronous(gpu_ctx):
    """Densities in and velocities out through page-locked host buffers with
    FTE_HOST_ASYNC (one stream synchronisation for all plans) give what the
    synchronising copies give."""
    import ctypes as C

    import torch

    ft = _ft()
    nv = 2
    plans, dens = [], []
    for i, (n, Lx, Ly) in enumerate([(3000, 1.0, 1.0), (5000, 2.0, 1.0), (2500, 1.0, 0.75)]):
        g = _geom(700 + i, n, Lx, Ly)
        f1s, f2s = _dens(750 + i, nv, n)
        plans.append(ft.Plan(i % 2, *g[:4], f1s[0], f2s[0], Lx, Ly, n1=g[4], n2=g[5], tol=1e-8, form=ft.FORM_MIXED,
                             nvmax=nv, ctx=gpu_ctx))
        dens.append((f1s, f2s))
    batch = ft.Batch(plans, nv, ctx=gpu_ctx)
    for i, (f1s, f2s) in enumerate(dens):
        batch.set_density(i, f1s, f2s)
    batch.launch(False)
    want = [batch.velocity(i) for i in range(len(plans))]
    pin_in = [(torch.tensor(np.ascontiguousarray(f1s)).pin_memory(), torch.tensor(np.ascontiguousarray(f2s)).pin_memory())
              for f1s, f2s in dens]
    pin_out = [(torch.zeros((nv, p.ntar), dtype=torch.float64).pin_memory(),
                torch.zeros((nv, p.ntar), dtype=torch.float64).pin_memory()) for p in plans]
    for i, (a, b) in enumerate(pin_in):
        batch.set_density(i, a.numpy(), b.numpy(), pinned_async=True)
    batch.launch(True)
    lib = ft.lib()
    for i, (u1, u2) in enumerate(pin_out):
        ft._check(lib.fte_batch_get_velocity(batch.h, i, C.c_void_p(u1.data_ptr()), C.c_void_p(u2.data_ptr()),
                                             ft.FTE_HOST_ASYNC))
    torch.cuda.synchronize()
    for i, (u1, u2) in enumerate(pin_out):
        assert rel_max(np.stack([u1.numpy(), u2.numpy()]), np.stack(want[i])) <= 1e-12, i
    batch.close()
    for p in plans:
        p.close()
