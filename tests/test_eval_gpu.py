"""GPU checks of the evaluation renderer (renderer.evaluation) and its metrics
(ff_image_metrics) against the oracle's restatement of the reference's rgb_ssim / PSNR."""
import math

import numpy as np
import pytest
import torch

from gpu_util import need_gpu
from oracle import ff_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    need_gpu()


@pytest.mark.parametrize("h,w,max_val", [(57, 83, 1.0), (11, 11, 1.0), (160, 120, 2.0)])
def test_image_metrics_match_oracle(h, w, max_val):
    from factor_fields_gb300.renderer import image_metrics
    rng = np.random.default_rng(h * w)
    a = rng.uniform(0, max_val, (h, w, 3)).astype(np.float32)
    a = np.cumsum(a, 1) / np.arange(1, w + 1)[None, :, None]  # some structure
    b = np.clip(a + rng.normal(0, 0.05 * max_val, a.shape), 0, max_val).astype(np.float32)
    a = a.astype(np.float32)
    mse, ssim = image_metrics(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), max_val)
    mse_r, ssim_r = O.image_metrics(a, b, max_val)
    assert abs(mse - mse_r) <= 1e-9 * mse_r
    assert abs(ssim - ssim_r) <= 1e-9
    _, one = image_metrics(torch.from_numpy(a).cuda(), torch.from_numpy(a).cuda(), max_val)
    assert abs(one - 1.0) < 1e-12


def test_evaluation_renders_whole_images():
    """evaluation() renders each image's rays in one pass; the PSNRs equal those of the
    reference-style chunked render (chunk 1,024) scored by the oracle, for the plain sampler
    and for the proposal sampler."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    from factor_fields_gb300.renderer import evaluation, render_ray
    from factor_fields_gb300.train import RadianceFieldTrainer
    scene = W.BlobScene(0)
    ds = scene.test_dataset([0, 3], width=64, height=48, n_steps=256)
    pool = torch.from_numpy(scene.ray_pool(1 << 14, 5, width=64, height=48)).float()
    gt = scene.render_gt(pool.double().numpy(), n_steps=256).cuda().float()
    pool = pool.cuda()
    torch.manual_seed(0)
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    sam = ProposalSampler(m)
    tr = RadianceFieldTrainer(m, sampler=sam, n_iters=100)
    g = torch.Generator(device="cuda").manual_seed(0)
    for _ in range(100):
        idx = torch.randint(0, pool.shape[0], (2048,), device="cuda", generator=g)
        tr.step(pool[idx], gt[idx])
    for use_sampler in (False, True):
        psnrs, extra = evaluation(ds, m, N_vis=-1, N_samples=512, white_bg=True,
                                  sampler=sam if use_sampler else None)
        assert len(psnrs) == 2 and len(extra["ssim"]) == 2 and len(extra["ms_per_image"]) == 2
        for k, idx in enumerate([0, 1]):
            rays = ds.all_rays[idx].cuda()
            if use_sampler:
                rgb, _ = sam.render(rays, is_train=False, white_bg=True)
            else:
                rgb, _ = render_ray(rays, m, chunk=1024, N_samples=512, white_bg=True)
            img = rgb.detach().clamp(0, 1).reshape(48, 64, 3).cpu().numpy()
            mse, ssim = O.image_metrics(img, ds.all_rgbs[idx].reshape(48, 64, 3).numpy())
            assert abs(psnrs[k] - (-10 * math.log10(mse))) < 1e-3
            assert abs(extra["ssim"][k] - ssim) < 1e-5
