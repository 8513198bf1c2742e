"""GPU input preparation (ProcessInputImages.fuseGroups for one group) against the CPU
restatement: affine-transformed views with linear interpolation, cosine blending, weighted
average and summed deconvolution weights.  Tolerance: 1e-5 relative on the fused image
(float interpolation), 1e-6 on the weights; voxels whose sample falls within 1e-9 of a
view's border (where double rounding may decide inside / outside) are excluded."""
import math

import numpy as np
import pytest

import mvrgb300 as M
import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def model(angle_deg, scale_z, t):
    a = math.radians(angle_deg)
    R = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    S = np.diag([1.0, 1.0, scale_z])
    return np.hstack([R @ S, np.asarray(t, dtype=np.float64).reshape(3, 1)])


@pytest.mark.parametrize("blend", [False, True])
def test_fuse_group_matches_oracle(blend):
    rng = np.random.default_rng(7)
    views = []
    for k, (ang, tz) in enumerate([(0.0, 0.0), (33.0, 4.0), (-61.0, -3.0)]):
        img = rng.uniform(0, 300, (20, 40, 48)).astype(np.float32)  # [z][y][x]
        m = model(ang, 1.5, (2.37 + k, -1.71, tz + 0.43))  # fractional: samples rarely land on a border
        v = {"img": img, "model": m}
        if k == 1:
            v["intensity"] = (1.37, -4.25)  # IntensityAdjuster of the second view
        if blend:
            v["fusion"] = ((2.0, 2.0, 1.0), (10.0, 10.0, 4.0))
            v["decon"] = ((1.0, 1.0, 0.5), (6.0, 6.0, 3.0))
        views.append(v)
    bb_min, bb_dims = (-10, -6, -14), (64, 44, 40)
    ref_img, ref_w = O.fuse_group(views, bb_min, bb_dims)
    dev = [torch.from_numpy(v["img"]).cuda() for v in views]
    out_i = torch.empty((bb_dims[2], bb_dims[1], bb_dims[0]), dtype=torch.float32, device="cuda")
    out_w = torch.empty_like(out_i)
    gv = []
    for v, d in zip(views, dev):
        g = {"img_ptr": d.data_ptr(), "dims": (v["img"].shape[2], v["img"].shape[1], v["img"].shape[0]),
             "model": v["model"], "intensity": v.get("intensity")}
        if blend:
            g["fusion"], g["decon"] = v["fusion"], v["decon"]
        gv.append(g)
    M.fuse_group(gv, bb_min, bb_dims, out_i.data_ptr(), out_w.data_ptr())
    img, w = out_i.cpu().numpy(), out_w.cpu().numpy()
    # voxels far from every view's border decision
    z, y, x = np.meshgrid(*[np.arange(n) for n in bb_dims[::-1]], indexing="ij")
    s = np.stack([x + bb_min[0], y + bb_min[1], z + bb_min[2]], -1).astype(np.float64)
    safe = np.ones(s.shape[:-1], bool)
    for v in views:
        inv = O._invert_affine(v["model"])
        t = s @ inv[:, :3].T + inv[:, 3]
        dims = np.array(v["img"].shape[::-1], dtype=np.float64)
        safe &= np.all((np.abs(t) > 1e-9) & (np.abs(t - (dims - 1)) > 1e-9), axis=-1)
    assert safe.mean() > 0.99
    assert np.abs(img - ref_img)[safe].max() <= 1e-5 * max(1.0, float(np.abs(ref_img).max()))
    assert np.abs(w - ref_w)[safe].max() <= 1e-6
    assert (ref_img > 0).mean() > 0.3  # the views cover a good part of the box
