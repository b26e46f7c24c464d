"""GPU checks of FusedAdam (ff_adam_step) against torch.optim.Adam."""
import pytest
import torch

from gpu_util import need_gpu, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    need_gpu()


def test_fused_adam_matches_torch_adam():
    """Five steps over two parameter groups (different learning rates), sizes that are not
    multiples of 4, one parameter that is an unaligned view; moments and parameters within
    float32 rounding (1e-5 relative) of torch's single-tensor Adam; the BF16 copies equal the rounded
    parameters; the gradients are zeroed."""
    from factor_fields_gb300.optim import FusedAdam
    gen = torch.Generator().manual_seed(0)
    sizes = [1, 7, 1024, 4097, 100003]
    base = torch.randn(sum(sizes) + 1, generator=gen)
    ref = [torch.nn.Parameter(t.clone().cuda()) for t in torch.split(base[1:], sizes)]
    holder = torch.randn(sizes[3] + 1, generator=gen).cuda()
    ours = [torch.nn.Parameter(t.detach().clone()) for t in ref]
    ours[3] = torch.nn.Parameter(holder[1:])  # storage offset 4 bytes: not 16-byte aligned
    with torch.no_grad():
        ours[3].copy_(ref[3])
    shadows = {p: torch.empty_like(p, dtype=torch.bfloat16) for p in ours[2:]}
    groups = lambda ps: [{"params": ps[:2], "lr": 2e-2}, {"params": ps[2:], "lr": 1e-3}]
    opt_ref = torch.optim.Adam(groups(ref), betas=(0.9, 0.99), eps=1e-8, foreach=False)
    opt = FusedAdam(groups(ours), betas=(0.9, 0.99), eps=1e-8, shadows=shadows)
    for it in range(5):
        for a, b in zip(ref, ours):
            g = torch.randn(a.shape, generator=gen).cuda() * (0.1 + it)
            a.grad = g.clone()
            b.grad = g.clone()
        opt_ref.step()
        opt.step()
        torch.cuda.synchronize()
        for a, b in zip(ref, ours):
            # float32 rounding: torch's kernels contract into FMAs, ff_adam_step rounds every
            # operation (a few ulp per step, accumulating over the steps)
            assert rel_err(b, a.detach()) < 1e-5
            sa, sb = opt_ref.state[a], opt.state[b]
            assert rel_err(sb["exp_avg"], sa["exp_avg"]) < 1e-5
            assert rel_err(sb["exp_avg_sq"], sa["exp_avg_sq"]) < 1e-5
            assert int(sb["step"]) == int(sa["step"]) == it + 1
            assert float(b.grad.abs().max()) == 0.0
        for p, s in shadows.items():
            assert torch.equal(s, p.detach().to(torch.bfloat16))


def test_trainer_with_fused_adam_trains_like_torch_adam():
    """Configuration 3 for 150 steps with FusedAdam (field and proposal) and with torch's Adam:
    the losses follow each other (float32 rounding and atomic order only) and go down."""
    import numpy as np
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    from factor_fields_gb300.train import RadianceFieldTrainer
    scene = W.BlobScene(0)
    pool = torch.from_numpy(scene.ray_pool(1 << 14, 5)).float()
    gt = scene.render_gt(pool.double().numpy(), n_steps=256).cuda().float()
    pool = pool.cuda()
    losses = {}
    for fused in (False, True):
        torch.manual_seed(0)
        m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
        tr = RadianceFieldTrainer(m, sampler=ProposalSampler(m, fused_adam=fused), n_iters=150, fused_adam=fused)
        g = torch.Generator(device="cuda").manual_seed(0)
        jit = torch.Generator(device="cuda").manual_seed(1)
        ls = []
        for it in range(150):
            idx = torch.randint(0, pool.shape[0], (2048,), device="cuda", generator=g)
            tr.jitter = torch.rand(2048, device="cuda", generator=jit)
            ls.append(float(tr.step(pool[idx], gt[idx])))
        losses[fused] = np.array(ls)
    first, last = losses[True][:20].mean(), losses[True][-20:].mean()
    assert last < 0.9 * first, (first, last)
    for a, b in ((0, 20), (65, 85), (130, 150)):
        fa, ta = losses[True][a:b].mean(), losses[False][a:b].mean()
        assert abs(fa - ta) < 0.05 * ta, (a, fa, ta)


def test_scheduled_adam_matches_host_schedule():
    """FusedAdam under its device schedule (ff_adam_step_scheduled: step count and learning rates
    in device memory, decayed on the device) against the host schedule (ff_adam_step): five steps
    with an lr decay after each, two groups; the moments agree exactly, the parameters to the
    rounding of the step size (float32 bias corrections on the device, double on the host), and
    sync_host() returns the host schedule's step counts and learning rates exactly."""
    from factor_fields_gb300.optim import FusedAdam
    gen = torch.Generator().manual_seed(1)
    sizes = [5, 1024, 4099]
    base = [torch.randn(s, generator=gen) for s in sizes]
    host = [torch.nn.Parameter(t.clone().cuda()) for t in base]
    devs = [torch.nn.Parameter(t.clone().cuda()) for t in base]
    groups = lambda ps: [{"params": ps[:1], "lr": 2e-2}, {"params": ps[1:], "lr": 1e-3}]
    opt_h = FusedAdam(groups(host), betas=(0.9, 0.99), eps=1e-8)
    opt_d = FusedAdam(groups(devs), betas=(0.9, 0.99), eps=1e-8)
    for p in host + devs:
        p.grad = torch.zeros_like(p)
    opt_d.enable_device_schedule()
    assert opt_d.device_schedule
    for it in range(5):
        for a, b in zip(host, devs):
            g = torch.randn(a.shape, generator=gen).cuda() * (0.5 + it)
            a.grad.copy_(g)
            b.grad.copy_(g)
        opt_h.step()
        opt_d.step()
        opt_h.decay_lr(0.93)
        opt_d.decay_lr(0.93)
    torch.cuda.synchronize()
    for a, b in zip(host, devs):
        # a few ulp of a step of at most lr = 2e-2 per step
        assert torch.allclose(a, b, rtol=1e-6, atol=1e-7)
        assert torch.allclose(opt_h.state[a]["exp_avg"], opt_d.state[b]["exp_avg"], rtol=0, atol=0)
        assert torch.allclose(opt_h.state[a]["exp_avg_sq"], opt_d.state[b]["exp_avg_sq"], rtol=0, atol=0)
        assert float(b.grad.abs().max()) == 0.0
    opt_d.sync_host()
    for gh, gd in zip(opt_h.param_groups, opt_d.param_groups):
        assert gh["lr"] == gd["lr"]  # the same float64 products
    for a, b in zip(host, devs):
        assert int(opt_d.state[b]["step"]) == int(opt_h.state[a]["step"]) == 5
    sd = opt_d.state_dict()  # synchronises first
    assert all(int(s["step"]) == 5 for s in sd["state"].values())


@pytest.mark.parametrize("proposal", [False, True])
def test_graph_step_with_update_trains_like_eager_step(proposal):
    """RadianceFieldTrainer.graph_step(optimize=True) (rendering, loss, backward and the fused
    Adam updates of field and proposal network in one CUDA graph, device schedule) against the
    eager step(optimize=True) from the same initial state on the same batches and jitter: the
    losses follow each other (atomic order only), and the step counts and decayed learning
    rates are the eager run's."""
    import numpy as np
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    from factor_fields_gb300.train import RadianceFieldTrainer
    scene = W.BlobScene(0)
    pool = torch.from_numpy(scene.ray_pool(1 << 14, 5)).float()
    gt = scene.render_gt(pool.double().numpy(), n_steps=256).cuda().float()
    pool = pool.cuda()
    iters, batch = 60, 2048
    out = {}
    for graph in (False, True):
        torch.manual_seed(0)
        m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
        if proposal:
            tr = RadianceFieldTrainer(m, sampler=ProposalSampler(m), n_iters=iters)
        else:
            m.cfg.renderer.density_shift = -4.0
            tr = RadianceFieldTrainer(m, n_samples=256, n_iters=iters)
        g = torch.Generator(device="cuda").manual_seed(0)
        jit = torch.Generator(device="cuda").manual_seed(1)
        tr.jitter = torch.empty(batch, device="cuda")  # refilled in place: the graph reads it
        ls = []
        for it in range(iters):
            idx = torch.randint(0, pool.shape[0], (batch,), device="cuda", generator=g)
            tr.jitter.copy_(torch.rand(batch, device="cuda", generator=jit))
            loss = tr.graph_step(pool[idx], gt[idx], optimize=True) if graph else tr.step(pool[idx], gt[idx])
            ls.append(float(loss))
        tr.opt.sync_host()
        out[graph] = (np.array(ls), [gr["lr"] for gr in tr.opt.param_groups],
                      sorted({int(s["step"]) for s in tr.opt.state.values()}))
        if proposal:
            tr.sampler.opt.sync_host()
            out[graph] += (sorted({int(s["step"]) for s in tr.sampler.opt.state.values()}),)
    (le, lre, ste, *pe), (lg, lrg, stg, *pg) = out[False], out[True]
    assert ste == stg == [iters] and lre == lrg
    if proposal:
        assert pe == pg == [[iters]]
    assert abs(lg[0] - le[0]) <= 1e-5 * le[0]  # the first step: same state, same batch
    for a, b in ((0, 10), (25, 35), (50, 60)):
        assert abs(lg[a:b].mean() - le[a:b].mean()) < 0.02 * le[a:b].mean(), (a, lg[a:b].mean(), le[a:b].mean())
    assert lg[-10:].mean() < lg[:10].mean()  # it trains


def test_graph_step_with_update_after_load_state_dict():
    """A load_state_dict of the optimizer drops its device schedule and replaces its moment
    buffers; the next graph_step(optimize=True) captures again and continues from the loaded
    step count and learning rates."""
    import copy
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.train import RadianceFieldTrainer
    scene = W.BlobScene(0)
    pool = torch.from_numpy(scene.ray_pool(1 << 12, 5)).float().cuda()
    gt = torch.rand(pool.shape[0], 3, device="cuda")
    torch.manual_seed(0)
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    m.cfg.renderer.density_shift = -4.0
    tr = RadianceFieldTrainer(m, n_samples=128, n_iters=50)
    rays, rgb = pool[:1024], gt[:1024]
    for _ in range(5):
        tr.graph_step(rays, rgb, optimize=True)
    sd = copy.deepcopy(tr.opt.state_dict())  # step 5
    lr5 = [g["lr"] for g in sd["param_groups"]]
    for _ in range(3):
        tr.graph_step(rays, rgb, optimize=True)
    tr.opt.load_state_dict(sd)
    assert not tr.opt.device_schedule
    loss = tr.graph_step(rays, rgb, optimize=True)  # captured again from the loaded state
    torch.cuda.synchronize()
    assert torch.isfinite(loss)
    tr.opt.sync_host()
    assert sorted({int(s["step"]) for s in tr.opt.state.values()}) == [6]
    for g, lr in zip(tr.opt.param_groups, lr5):
        assert g["lr"] == lr * tr.lr_factor
