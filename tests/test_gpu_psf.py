"""GPU PSF preparation (PSFExtraction / PSFCombination / PSFPreparation) against the CPU
restatement.  The extraction, averaging, resizing and projections repeat the reference's
float and double operations in the same order and must agree bit for bit; the normalised
transformed PSFs agree to 1e-7 (values in [0, 1])."""
import math

import numpy as np
import pytest

import mvrgb300 as M
import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def xyz(a):
    return (a.shape[2], a.shape[1], a.shape[0])


def empty(d):
    return torch.empty((d[2], d[1], d[0]), dtype=torch.float32, device="cuda")


def model(ay, az, scale, t):
    a, b = math.radians(ay), math.radians(az)
    Ry = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    Rz = np.array([[math.cos(b), -math.sin(b), 0], [math.sin(b), math.cos(b), 0], [0, 0, 1]])
    return np.hstack([Rz @ Ry @ np.diag(scale), np.asarray(t, dtype=np.float64).reshape(3, 1)])


def test_extract_matches_oracle_bitwise():
    rng = np.random.default_rng(3)
    img = rng.uniform(0, 100, (30, 41, 52)).astype(np.float32)
    # fractional bead positions, some near the faces so that the neighbourhoods wrap
    loc = np.stack([rng.uniform(-3, 55, 40), rng.uniform(-3, 44, 40), rng.uniform(-3, 33, 40)], axis=1)
    size = (9, 11, 13)
    ref = O.psf_extract(img, loc, size)
    out = empty(size)
    M.psf_extract(dev(img).data_ptr(), xyz(img), loc, size, out.data_ptr())
    got = out.cpu().numpy()
    assert np.array_equal(got, ref)
    M.psf_extract(dev(img).data_ptr(), xyz(img), np.zeros((0, 3)), size, out.data_ptr())
    assert not out.cpu().numpy().any()


@pytest.mark.parametrize("m", [model(0, 90, (1, 1, 1), (0, 0, 0)), model(35, 20, (1, 1, 2.5), (3.2, -1.1, 7.9)),
                               model(-50, 0, (0.5, 0.5, 1.3), (0, 0, 0))])
def test_transform_normalized_matches_oracle(m):
    rng = np.random.default_rng(5)
    psf = rng.gamma(2.0, 1.0, (15, 11, 13)).astype(np.float32)
    ref = O.psf_transform_normalized(psf, m)
    d = M.psf_transformed_dims(xyz(psf), m)
    assert d == xyz(ref)
    src = dev(psf)
    out = empty(d)
    M.psf_transform_normalized(src.data_ptr(), xyz(psf), m, out.data_ptr(), d)
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-7
    assert np.array_equal(src.cpu().numpy(), psf)  # the input PSF is left unchanged


def test_combination_matches_oracle_bitwise():
    rng = np.random.default_rng(8)
    psfs = [rng.random((9, 7, 11)).astype(np.float32), rng.random((13, 9, 7)).astype(np.float32),
            rng.random((11, 11, 9)).astype(np.float32)]
    ds = [dev(p) for p in psfs]
    for mx in (True, False):
        ref = O.psf_average(psfs, max_size=mx)
        out = empty(M.psf_average_dims([xyz(p) for p in psfs], mx))
        got_dims = M.psf_average([t.data_ptr() for t in ds], [xyz(p) for p in psfs], mx, out.data_ptr())
        assert got_dims == xyz(ref)
        assert np.array_equal(out.cpu().numpy(), ref)
    size = (15, 12, 17)
    out = empty(size)
    M.psf_make_same_size(ds[0].data_ptr(), xyz(psfs[0]), size, out.data_ptr())
    assert np.array_equal(out.cpu().numpy(), O.psf_make_same_size(psfs[0], size))
    for dim, use_max in ((-1, True), (0, False), (1, True), (2, False)):
        ref, rd = O.psf_projection(psfs[1], dim, use_max)
        out = torch.empty(ref.size, dtype=torch.float32, device="cuda")
        used = M.psf_projection(ds[1].data_ptr(), xyz(psfs[1]), dim, use_max, out.data_ptr())
        assert used == rd
        assert np.array_equal(out.cpu().numpy().reshape(ref.shape), ref)
    t = dev(psfs[2])
    M.psf_remove_min_projections(t.data_ptr(), xyz(psfs[2]))
    assert np.array_equal(t.cpu().numpy(), O.psf_remove_min_projections(psfs[2]))


def test_load_group_transform_psfs_matches_oracle():
    rng = np.random.default_rng(11)
    base = rng.gamma(2.0, 1.0, (21, 9, 9)).astype(np.float32)
    groups = [[(base, model(0, 0, (1, 1, 1), (0, 0, 0))), (base[::-1].copy(), model(180, 0, (1, 1, 1), (5, 0, 2)))],
              [(base, model(90, 0, (1, 1, 1), (0, 0, 0)))],
              [(base, model(45, 10, (1, 1, 1.5), (1, 2, 3))), (base, model(47, 12, (1, 1, 1.5), (1, 2, 3)))]]
    for same in (True, False):
        ref = O.load_group_transform_psfs(groups, same)
        got = M.load_group_transform_psfs(groups, same)
        assert [g.shape for g in got] == [r.shape for r in ref]
        for g, r in zip(got, ref):
            assert np.abs(g - r).max() <= 1e-7


def test_psf_errors():
    sing = np.zeros((3, 4))
    with pytest.raises(M.MvrError):
        M.psf_transformed_dims((5, 5, 5), np.full((3, 4), np.nan))
    t = dev(np.ones((5, 5, 5)))
    with pytest.raises(M.MvrError):
        M.psf_transform_normalized(t.data_ptr(), (5, 5, 5), sing, t.data_ptr(), (1, 1, 1))
    with pytest.raises(M.MvrError):
        M.psf_extract(t.data_ptr(), (5, 5, 5), [(1, 1, 1)], (0, 5, 5), t.data_ptr())
