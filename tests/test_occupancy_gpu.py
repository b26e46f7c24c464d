"""GPU parity of the occupancy-volume maintenance (ff_occupancy_mask, FactorFields.updateAlphaMask)
against the oracle: bit-exact bitfields, volumes and bounding boxes (integer / boolean work)."""
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


def blob_volume(shape, seed, n_blobs=6, n_floaters=40):
    """Gaussian blobs of several sizes, isolated bright voxels (floaters), values outside [0, 1]."""
    rng = np.random.default_rng(seed)
    d, h, w = shape
    z, y, x = np.meshgrid(np.arange(d), np.arange(h), np.arange(w), indexing="ij")
    a = np.zeros(shape, np.float64)
    for _ in range(n_blobs):
        c = rng.uniform(0, 1, 3) * [d, h, w]
        s = rng.uniform(0.5, 0.12 * min(shape) + 1.0)
        a += rng.uniform(0.5, 2.0) * np.exp(-(((z - c[0]) ** 2 + (y - c[1]) ** 2 + (x - c[2]) ** 2) / (2 * s * s)))
    idx = rng.integers(0, a.size, n_floaters)
    a.reshape(-1)[idx] = rng.uniform(0.2, 1.5, n_floaters)
    a -= 0.05  # some negative values (clamped to 0)
    return a.astype(np.float32)


def run_native(alpha, threshold, min_size):
    from factor_fields_gb300 import _native as N
    d, h, w = alpha.shape
    need = int(N.lib().ff_occupancy_workspace_bytes(d, h, w))
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    a = torch.from_numpy(alpha).cuda()
    bits = torch.full(((alpha.size + 31) // 32,), -7, dtype=torch.int32, device="cuda")
    vol = torch.empty(alpha.shape, device="cuda")
    bbox = torch.empty(6, dtype=torch.int32, device="cuda")
    N.call("ff_occupancy_mask", N.ptr(a), d, h, w, threshold, min_size, N.ptr(bits), N.ptr(vol), N.ptr(bbox),
           N.ptr(ws), need, N.stream_ptr())
    return bits.cpu().numpy(), vol.cpu().numpy(), bbox.cpu().numpy()


@pytest.mark.parametrize("shape,threshold,min_size", [((37, 41, 29), 0.3, None), ((16, 16, 16), 0.5, 1),
                                                      ((128, 128, 128), 0.08, None), ((5, 70, 9), 0.2, 3)])
def test_occupancy_mask_matches_oracle(shape, threshold, min_size):
    alpha = blob_volume(shape, seed=sum(shape))
    if min_size is None:
        min_size = int(math.ceil(np.mean(shape)))  # what updateAlphaMask passes
    bits, vol, bbox = run_native(alpha, threshold, min_size)
    occ, words, box = O.occupancy_mask(alpha, threshold, min_size)
    assert np.array_equal(bits, words)
    assert np.array_equal(vol > 0.5, occ) and set(np.unique(vol)) <= {0.0, 1.0}
    assert box is not None and tuple(int(v) for v in bbox) == tuple(int(v) for v in box)
    if min_size > 27:  # the filter removed something the threshold alone kept (a pooled floater: <= 27 voxels)
        occ0, _, _ = O.occupancy_mask(alpha, threshold, 1)
        assert occ0.sum() > occ.sum()


def test_occupancy_mask_empty_volume():
    bits, vol, bbox = run_native(np.zeros((8, 9, 10), np.float32), 0.5, 4)
    assert not bits.any() and not vol.any()
    assert bbox[0] > bbox[3]


def test_update_alpha_mask_uses_the_native_pipeline(monkeypatch):
    """updateAlphaMask on a given dense alpha: the mask bits, the 0/1 volume and the new aabb
    (padded bounding box of the kept voxel centres, models/FactorFields.py:776-790)."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    shape = (48, 40, 44)  # (Z, Y, X) of a (44, 40, 48) grid
    alpha = blob_volume(shape, seed=3)
    grid = (shape[2], shape[1], shape[0])
    _, dense_xyz = FactorFields.getDenseAlpha(m, grid, times=1)
    monkeypatch.setattr(m, "getDenseAlpha", lambda *a, **k: (torch.from_numpy(alpha).cuda(), dense_xyz))
    new_aabb = m.updateAlphaMask(grid, is_update_alphaMask=True)
    thres = float(m.cfg.renderer.alphaMask_thres)
    occ, words, _ = O.occupancy_mask(alpha, thres, int(math.ceil(np.mean(shape))))
    assert np.array_equal(m.alphaMask.bits.cpu().numpy(), words)
    assert np.array_equal(m.alphaMask.alpha_volume.view(shape).cpu().numpy() > 0.5, occ)
    xyz = dense_xyz.cpu().numpy()[occ]
    lo, hi = xyz.min(0), xyz.max(0)
    pad = (hi - lo) / 20
    assert np.allclose(new_aabb.cpu().numpy(), np.stack([lo - pad, hi + pad]), rtol=0, atol=1e-6)


def _model_with_mask(seed=4, reso=(40, 36, 44)):
    """cfg2 model with an alpha mask from a thresholded blob volume over its aabb."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.renderer import AlphaGridMask
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    vol = (blob_volume(reso, seed=seed, n_blobs=3, n_floaters=10) > 0.6).astype(np.float32)
    m.alphaMask = AlphaGridMask(m.device, m.inward_aabb, torch.from_numpy(vol).cuda())
    return m, vol


@pytest.mark.parametrize("bbox_only", [False, True])
def test_filtering_rays_matches_oracle(bbox_only):
    """filtering_rays (models/FactorFields.py:825-841): a ray survives if any of its 256
    un-jittered samples has trilinear occupancy > 0 (or, bbox_only, if it meets the box);
    survivors keep their order. Rays from the blob scene's cameras plus rays that miss."""
    from factor_fields_gb300 import workloads as W
    m, vol = _model_with_mask()
    rays = W.BlobScene(0).ray_pool(3000, 7).astype(np.float32)
    rng = np.random.default_rng(8)
    miss = np.concatenate([rng.uniform(3, 4, (500, 3)), np.tile([[1.0, 0.0, 0.0]], (500, 1))], 1).astype(np.float32)
    rays = np.concatenate([rays, miss])[rng.permutation(3500)]
    rgbs = rng.uniform(0, 1, (rays.shape[0], 3)).astype(np.float32)
    kept_r, kept_c = m.filtering_rays(torch.from_numpy(rays).cuda(), torch.from_numpy(rgbs).cuda(), N_samples=256,
                                      chunk=1024, bbox_only=bbox_only)
    aabb = m.aabb.cpu().numpy()
    if bbox_only:
        o, d = rays[:, :3], rays[:, 3:6]
        vec = np.where(d == 0, np.float32(1e-6), d)
        ra = ((aabb[1] - o) / vec).astype(np.float32)
        rb = ((aabb[0] - o) / vec).astype(np.float32)
        keep = np.minimum(ra, rb).max(-1) < np.maximum(ra, rb).min(-1)
    else:
        xyz, _, _ = O.sample_point(rays[:, :3], rays[:, 3:6], aabb, float(m.stepSize), 256)
        hit = O.occupancy_test(vol, m.alphaMask.aabb.cpu().numpy(), xyz.reshape(-1, 3), thres=0.0)
        keep = hit.reshape(rays.shape[0], 256).any(-1)
    assert 0 < keep.sum() < rays.shape[0]
    assert np.array_equal(kept_r.cpu().numpy(), rays[keep])
    assert np.array_equal(kept_c.cpu().numpy(), rgbs[keep])


def test_shrink_rebuilds_the_field_for_the_new_box():
    """shrink (models/FactorFields.py:795-809): new aabb, grids re-derived for it (setup_params)
    and re-initialised, render step recomputed; rendering works afterwards."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.config import FieldGeometry
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    new_aabb = torch.tensor([[-1.0, -0.8, -0.5], [0.9, 1.1, 0.7]])
    m.shrink(new_aabb)
    assert torch.equal(m.aabb.cpu(), new_aabb) and torch.equal(m.inward_aabb.cpu(), new_aabb)
    g = FieldGeometry(m.cfg)
    assert list(m.coeff_reso) == list(g.coeff_reso) and list(m.basis_reso) == list(g.basis_reso)
    assert m.coeff_flat.numel() == m.layout.coeff_numel
    assert torch.all(m.coeffs[0] == float(m.cfg.model.coef_init))
    size = (new_aabb[1] - new_aabb[0])
    units = size / (m.gridSize.cpu().float() - 1)
    assert abs(float(m.stepSize) - float(units.mean() * m.cfg.renderer.step_ratio)) < 1e-6
    rays = torch.from_numpy(W.BlobScene(0).ray_pool(256, 2)).float().cuda()
    rgb, depth, _ = m(rays, white_bg=True, is_train=False, N_samples=256)
    assert torch.isfinite(rgb).all() and rgb.shape == (256, 3)
