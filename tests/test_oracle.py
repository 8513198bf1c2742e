"""The CPU oracle against the golden fixtures (independent numpy restatement),
direct spatial convolution and analytic known-answer cases."""
import itertools
import os

import numpy as np
import pytest

import oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 8, 12, 13, 31, 96, 97, 124, 156, 192, 222, 252])
def test_fft1d_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    assert np.abs(O.fft1d(x) - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    assert np.abs(O.fft1d(x, inverse=True) - np.fft.ifft(x) * n).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_mirror_single_ramp():
    # imglib2 extendMirrorSingle: border voxel not repeated, period 2n-2
    n = 5
    got = [O.mirror_single(i, n) for i in range(-9, 14)]
    exp = [1, 0, 1, 2, 3, 4, 3, 2, 1, 0, 1, 2, 3, 4, 3, 2, 1, 0, 1, 2, 3, 4, 3]
    assert got == exp
    assert O.mirror_single(-3, 1) == 0


def _direct(blk, k, ext, val):
    bz, by, bx = blk.shape
    kz, ky, kx = k.shape
    out = np.zeros(blk.shape)
    for z, y, x in itertools.product(range(bz), range(by), range(bx)):
        s = 0.0
        for tz, ty, tx in itertools.product(range(kz), range(ky), range(kx)):
            g = (z - (tz - kz // 2), y - (ty - ky // 2), x - (tx - kx // 2))
            if 0 <= g[0] < bz and 0 <= g[1] < by and 0 <= g[2] < bx:
                v = blk[g]
            elif ext == O.EXT_MIRROR_SINGLE:
                v = blk[O.mirror_single(g[0], bz), O.mirror_single(g[1], by), O.mirror_single(g[2], bx)]
            elif ext == O.EXT_VALUE:
                v = val
            else:
                v = 0.0
            s += v * k[tz, ty, tx]
        out[z, y, x] = s
    return out


@pytest.mark.parametrize("ext", [O.EXT_ZERO, O.EXT_MIRROR_SINGLE, O.EXT_VALUE])
def test_convolution_vs_direct(ext):
    rng = np.random.default_rng(3)
    blk = rng.random((4, 5, 6)).astype(np.float32)
    k = rng.random((3, 4, 5)).astype(np.float32)  # even size along y
    got = O.convolve(blk, k, ext, 1.0)
    ref = _direct(blk.astype(np.float64), k.astype(np.float64), ext, 1.0)
    assert np.abs(got - ref).max() < 1e-12


def test_convolution_golden():
    g = np.load(os.path.join(G, "conv_cases.npz"))
    for name, k, ext in [("mirror_odd", "k_odd", 1), ("value_odd", "k_odd", 2), ("zero_odd", "k_odd", 0),
                         ("mirror_even", "k_even", 1), ("value_even", "k_even", 2)]:
        assert np.abs(O.convolve(g["block"], g[k], ext, 1.0) - g[name]).max() < 1e-10, name


def test_block_seq_golden():
    b = np.load(os.path.join(G, "block_cases.npz"))
    out, st = O.block_seq(b["psi"], b["img0"], b["w0"], b["k1_0"], b["k2_0"], float(b["lam"]), 1e-4,
                          float(b["max"][0]))
    assert np.array_equal(out, b["seq_out"])  # float-faithful path is bit-exact
    assert np.allclose(st, b["seq_stats"], rtol=1e-12)
    out, st = O.block_seq(b["psi"], b["img0"], b["w0"], b["k1_0"], b["k2_0"], float(b["lam"]), 1e-4,
                          float(b["max"][0]), fp64=True)
    assert rel_l2(out, b["seq_out64"]) < 1e-12
    assert np.allclose(st, b["seq_stats64"], rtol=1e-10)


def test_block_mul_golden():
    b = np.load(os.path.join(G, "block_cases.npz"))
    args = ([b["img0"], b["img1"]], [b["w0"], b["w1"]], [b["k1_0"], b["k1_1"]], [b["k2_0"], b["k2_1"]],
            float(b["lam"]), 1e-4, b["max"])
    out, st = O.block_mul(b["psi"], *args)
    assert np.array_equal(out, b["mul_out"])
    assert np.allclose(st, b["mul_stats"], rtol=1e-12)
    out, st = O.block_mul(b["psi"], *args, fp64=True)
    assert rel_l2(out, b["mul_out64"]) < 1e-12


@pytest.mark.parametrize("psf_type", [0, 1, 2, 3])
def test_psf_init_golden(psf_type):
    p = np.load(os.path.join(G, "psf_cases.npz"))
    k1, k2 = O.psf_init([p["raw0"], p["raw1"], p["raw2"]], psf_type, 4)
    for v in range(3):
        assert np.array_equal(k1[v], p[f"t{psf_type}_k1_{v}"])
        ref = p[f"t{psf_type}_k2_{v}"]
        assert np.abs(k2[v] - ref).max() <= 1e-6 * np.abs(ref).max()


def test_invert_even_quirk():
    p = np.load(os.path.join(G, "psf_cases.npz"))
    assert np.array_equal(O.invert_kernel(p["even"]), p["even_inv"])
    odd = np.arange(3 * 5 * 7, dtype=np.float32).reshape(7, 5, 3)
    assert np.array_equal(O.invert_kernel(odd), odd[::-1, ::-1, ::-1])


def test_norm_to_sum1_double_counts_first_portion():
    k = np.ones(100, dtype=np.float32)
    # T = 4: first portion = 25 voxels counted twice -> sum 125
    assert np.allclose(O.norm_to_sum1(k, 4), 1.0 / 125.0)
    assert np.allclose(O.norm_to_sum1(k, 0), 1.0 / 100.0)


def test_weights_and_psi_init_golden():
    v = np.load(os.path.join(G, "volume_cases.npz"))
    ws = O.normalize_weights([v["raw_w0"], v["raw_w1"]])
    assert np.array_equal(ws[0], v["w0"]) and np.array_equal(ws[1], v["w1"])
    psi, mx, avg = O.psi_init_avg([v["img0"], v["img1"]])
    assert abs(avg - float(v["avg"])) < 1e-9 * abs(avg)
    assert np.array_equal(mx, v["max"])
    assert np.all(psi == np.float32(avg))


def test_block_geometry():
    # 256^3, k = 31x31x61 -> doubled 61x61x121, block 192^3 -> effective 132x132x72, 2x2x4 blocks
    bl = O.divide_into_blocks((256, 256, 256), (61, 61, 121), (192, 192, 192))
    assert len(bl) == 16
    assert bl[0]["eff_size"] == (132, 132, 72) and bl[0]["offset"] == (-30, -30, -60)
    assert bl[-1]["eff_offset"] == (132, 132, 216) and bl[-1]["eff_size"] == (124, 124, 40)
    assert O.divide_into_blocks((10, 10, 10), (11, 3, 3), (10, 10, 10)) is None
    # fewest blocks per slab: products (8, 8, 4) -> slabs along z
    assert O.sort_dim((2, 2, 4), 1) == 2
    # equal products keep the last dimension (HashMap overwrite)
    assert O.sort_dim((2, 2, 2), 1) == 2
    assert O.sort_dim((3, 1, 1), 1) == 0


@pytest.mark.parametrize("mul,key,bs,lam", [(False, "seq", (28, 28, 28), None), (True, "mul", (28, 28, 28), None),
                                            (False, "one", (48, 44, 48), 0.0)])
def test_volume_runs_golden(mul, key, bs, lam):
    v = np.load(os.path.join(G, "volume_cases.npz"))
    lam = float(v["lam"]) if lam is None else lam
    out, st = O.decon_run(v["psi0"], [v["img0"], v["img1"]], [v["w0"], v["w1"]], [v["k1_0"], v["k1_1"]],
                          [v["k2_0"], v["k2_1"]], bs, 2, mul=mul, lam=lam, max_intensities=v["max"])
    assert np.array_equal(out, v[key + "_psi"])
    assert np.allclose(st, v[key + "_stats"], rtol=1e-10)


def test_volume_fp64_golden():
    v = np.load(os.path.join(G, "volume_cases.npz"))
    out, _ = O.decon_run(v["psi0"], [v["img0"], v["img1"]], [v["w0"], v["w1"]], [v["k1_0"], v["k1_1"]],
                         [v["k2_0"], v["k2_1"]], (28, 28, 28), 2, lam=float(v["lam"]),
                         max_intensities=v["max"], fp64=True)
    assert rel_l2(out, v["seq_psi64"]) < 1e-12


def test_kat_delta_psf_identity():
    # delta PSF: both convolutions are the identity, so psi' = img where img > 0 (lambda 0, w 1)
    rng = np.random.default_rng(5)
    img = rng.uniform(1, 50, (6, 7, 8)).astype(np.float32)
    img[0, 0, :3] = 0
    psi = rng.uniform(1, 50, img.shape).astype(np.float32)
    d = np.ones((1, 1, 1), np.float32)
    out, _ = O.block_seq(psi, img, np.ones_like(img), d, d, 0.0, 1e-4, 100.0)
    m = img > 0
    assert np.allclose(out[m], img[m], rtol=4e-6)  # float rounding of psi + (next - psi) * w
    assert np.array_equal(out[~m], psi[~m])  # ratio 1 outside the data


def test_kat_constant_fixed_point():
    c = 37.0
    img = np.full((10, 12, 14), c, np.float32)
    k = np.random.default_rng(1).random((3, 5, 5)).astype(np.float32)
    k /= k.sum()
    k2 = O.invert_kernel(k)
    out, _ = O.block_seq(img.copy(), img, np.ones_like(img), k, k2, 0.0, 1e-4, c)
    assert np.abs(out - c).max() < 1e-4


def test_kat_guards():
    # psi * conv2 <= 0 -> minValue; w = 0 keeps psi; NaN never escapes
    psi = np.full((3, 3, 3), 5.0, np.float32)
    img = np.zeros_like(psi)  # ratio 1 everywhere -> conv2 = 1
    d = np.ones((1, 1, 1), np.float32)
    w = np.ones_like(psi)
    w[0] = 0
    out, st = O.block_seq(psi, img, w, d, d, 0.0, 1e-4, 10.0)
    assert np.array_equal(out, psi)
    assert st == (0.0, 0.0)
    neg = np.full_like(psi, -1.0)
    out, st = O.block_seq(neg, img, np.ones_like(psi), d, d, 0.0, 1e-4, 10.0)
    assert np.allclose(out, 1e-4, rtol=0, atol=1e-7)  # -1 + (1e-4 - (-1)) * 1 in float


def test_seq_equals_mul_for_one_view():
    b = np.load(os.path.join(G, "block_cases.npz"))
    a, sa = O.block_seq(b["psi"], b["img0"], b["w0"], b["k1_0"], b["k2_0"], 0.0, 1e-4, float(b["max"][0]))
    m, sm = O.block_mul(b["psi"], [b["img0"]], [b["w0"]], [b["k1_0"]], [b["k2_0"]], 0.0, 1e-4, [b["max"][0]])
    assert np.array_equal(a, m)
    assert np.allclose(sa, sm)


def test_gauss3_kernel_and_known_answers():
    # Gauss3 half kernel: size max(2, (int)(3 sigma + 0.5) + 1), normalised to sum 1
    for sigma in (0.5, 1.0, 2.0, 5.0):
        h = O.gauss3_half_kernel(sigma)
        assert len(h) == max(2, int(3 * sigma + 0.5) + 1)
        assert abs(h[0] + 2 * h[1:].sum() - 1.0) < 1e-14
    # a constant volume is a fixed point, an interior delta gives the separable kernel
    assert np.abs(O.gauss3(np.full((7, 9, 11), 4.0), 1.5) - 4.0).max() < 1e-12
    v = np.zeros((31, 31, 31))
    v[15, 15, 15] = 1.0
    h = O.gauss3_half_kernel(2.0)
    full = np.concatenate([h[:0:-1], h])
    g = O.gauss3(v, 2.0)
    c = len(h) - 1
    assert np.allclose(g[15, 15, 15 - c:15 + c + 1], full * full[c] * full[c], atol=1e-15)
    # mirror-single at the border (period 2n - 2, the edge voxel not repeated): a delta at
    # x = 1 is seen twice from x = 0 (offsets -1 and +1) and at x = 1 also through x = -1 -> 1;
    # a delta at x = 0 is seen once from x = 1
    h = O.gauss3_half_kernel(1.0)
    v = np.zeros((1, 1, 12))
    v[0, 0, 1] = 1.0
    g = O.gauss3(v, 1.0)
    assert abs(g[0, 0, 0] - 2 * h[1]) < 1e-15 and abs(g[0, 0, 1] - (h[0] + h[2])) < 1e-15
    v = np.zeros((1, 1, 12))
    v[0, 0, 0] = 1.0
    g = O.gauss3(v, 1.0)
    assert abs(g[0, 0, 1] - h[1]) < 1e-15 and abs(g[0, 0, 0] - h[0]) < 1e-15


def test_psi_init_known_answers():
    rng = np.random.default_rng(3)
    shape = (8, 10, 12)
    a = rng.uniform(1, 5, shape).astype(np.float32)
    # one view with weight 1: the fusion is the image itself, blurred
    psi, mx, avg = O.psi_init_blurred_fused([a], [np.ones(shape, np.float32)], 1.0)
    assert np.allclose(psi, O.gauss3(a, 1.0), rtol=1e-6)
    assert mx[0] == a.max() and abs(avg - a.astype(np.float64).mean()) < 1e-9
    # views without data (0) do not count; zero weight everywhere gives 0
    z = np.zeros(shape, np.float32)
    psi, mx, avg = O.psi_init_blurred_fused([a, z], [np.ones(shape, np.float32)] * 2, 1.0)
    assert mx[1] == 0.0 and abs(avg - a.astype(np.float64).mean()) < 1e-9
    psi, _, _ = O.psi_init_blurred_fused([a], [z], 1.0)
    assert np.all(psi == 0.0)
    # approximate average: the y-z slice at x = nx / 2
    psi, mx, avg = O.psi_init_avg_approx([a, 2 * a])
    sl = a[:, :, 6].astype(np.float64)
    assert abs(avg - 1.5 * sl.mean()) < 1e-9 and mx[1] == np.float32(2 * sl.max())
    assert np.all(psi == np.float32(avg))


def test_fusion_known_answers():
    # identity model, no blending: interior voxels are max(1, img); the view's border voxels
    # are not strictly inside it and read the outside value 0 (intersectsLinearInterpolation)
    rng = np.random.default_rng(0)
    img = rng.uniform(0, 5, (6, 7, 8)).astype(np.float32)
    ident = np.hstack([np.eye(3), np.zeros((3, 1))])
    im, w = O.fuse_group([{"img": img, "model": ident}], (0, 0, 0), (8, 7, 6))
    assert np.array_equal(im[1:-1, 1:-1, 1:-1], np.maximum(1, img[1:-1, 1:-1, 1:-1]))
    assert im[0].max() == 0 and im[:, :, -1].max() == 0 and np.all(w == 1)
    # a half-voxel shift interpolates linearly between neighbours
    shift = ident.copy()
    shift[0, 3] = -0.5
    im, _ = O.fuse_group([{"img": img, "model": shift}], (0, 0, 0), (8, 7, 6))
    mid = 0.5 * (img[2, 3, 3].astype(np.float64) + img[2, 3, 4])
    assert abs(im[2, 3, 3] - max(1.0, mid)) < 1e-6
    # blending: 0 within the border, (cos((1 - d) pi) + 1) / 2 over the range, 1 beyond
    lut = O.blending_lut()
    assert lut[0] == 0 and abs(lut[500] - 0.5) < 1e-12 and lut[1000] == 1
    loc = np.array([[1.0, 20, 20], [2.0 + 5.0, 20, 20], [20, 20, 20]], dtype=np.float32)
    wts = O.blending_weight(loc, (41, 41, 41), (2, 2, 2), (10, 10, 10))
    assert wts[0] == 0 and abs(wts[1] - 0.5) < 1e-6 and wts[2] == 1
    # two views with complementary blending average with their weights; the deconvolution
    # weight is the plain sum
    # intensity adjustment v m00 + m01 (double, stored as float) before the interpolation
    im, _ = O.fuse_group([{"img": img, "model": ident, "intensity": (2.5, 3.0)}], (0, 0, 0), (8, 7, 6))
    adj = (img.astype(np.float64) * 2.5 + 3.0).astype(np.float32)
    assert np.array_equal(im[1:-1, 1:-1, 1:-1], np.maximum(1, adj[1:-1, 1:-1, 1:-1]))
    im, w = O.fuse_group([{"img": img, "model": ident}, {"img": 3 * img, "model": ident}], (0, 0, 0), (8, 7, 6))
    assert np.allclose(im[1:-1, 1:-1, 1:-1], 0.5 * (np.maximum(1, img) + np.maximum(1, 3 * img))[1:-1, 1:-1, 1:-1],
                       rtol=1e-6)
    assert np.all(w == 2)


def test_psf_extraction_known_answers():
    # a single bead: at an integer location the neighbourhood is the bead itself; half a voxel
    # off it splits linearly; several locations add up; the image wraps periodically
    img = np.zeros((20, 22, 24), np.float32)
    img[10, 11, 12] = 8
    p = O.psf_extract(img, [(12, 11, 10)], (5, 5, 5))
    assert p[2, 2, 2] == 8 and p.sum() == 8
    p = O.psf_extract(img, [(12.5, 11, 10)], (5, 5, 5))
    assert p[2, 2, 2] == 4 and p[2, 2, 1] == 4 and p.sum() == 8
    p = O.psf_extract(img, [(12, 11, 10), (12, 11, 10)], (5, 5, 5))
    assert p[2, 2, 2] == 16
    edge = np.zeros((20, 22, 24), np.float32)
    edge[0, 0, 0] = 3
    p = O.psf_extract(edge, [(0, 0, 0)], (5, 5, 5))
    assert p[2, 2, 2] == 3 and p.sum() == 3
    p = O.psf_extract(edge, [(23, 21, 19)], (5, 5, 5))  # the bead one voxel beyond, wrapped
    assert p[3, 3, 3] == 3
    assert not O.psf_extract(img, [], (5, 5, 5)).any()  # no detections: a zero PSF


def test_psf_transform_known_answers():
    rng = np.random.default_rng(0)
    q = rng.random((7, 5, 9)).astype(np.float32)
    n = O.psf_normalize(q)
    assert n.min() == 0 and n.max() == 1
    # identity: the normalised PSF itself
    ident = np.hstack([np.eye(3), np.zeros((3, 1))])
    assert O.psf_transformed_geometry((9, 5, 7), ident)[0] == (9, 5, 7)
    assert np.array_equal(O.psf_transform_normalized(q, ident), n)
    # a translation does not move the PSF (its centre stays the centre)
    shifted = ident.copy()
    shifted[:, 3] = (10.0, -3.0, 7.0)
    assert np.array_equal(O.psf_transform_normalized(q, shifted), n)
    # 90 degrees about z: (x, y, z) -> (-y, x, z); sizes swap, values rotate exactly
    rot = np.array([[0, -1, 0, 0], [1, 0, 0, 0], [0, 0, 1, 0]], dtype=np.float64)
    size, off = O.psf_transformed_geometry((9, 5, 7), rot)
    assert size == (5, 9, 7) and np.array_equal(off, [-4, 0, 0])
    t = O.psf_transform_normalized(q, rot)
    z, y, x = np.meshgrid(np.arange(7), np.arange(9), np.arange(5), indexing="ij")
    assert np.array_equal(t, n[z, 4 - x, y])
    # an even extent becomes odd: scaling x by 1.5 gives extent 12 -> 13 voxels
    sc = ident.copy()
    sc[0, 0] = 1.5
    assert O.psf_transformed_geometry((9, 5, 7), sc)[0] == (13, 5, 7)


def test_psf_combination_known_answers():
    a = np.arange(27, dtype=np.float32).reshape(3, 3, 3)
    b = np.ones((5, 3, 1), np.float32)  # x 1, y 3, z 5
    # centred average on the largest size: b's single x column sits at x = 1
    avg = O.psf_average([a, b], max_size=True)
    assert avg.shape == (5, 3, 3)
    assert avg[0, 1, 1] == np.float32(0.5) and avg[0, 1, 0] == 0
    assert avg[2, 1, 1] == np.float32((13 + 1) / 2)
    # smallest size: 1 x 3 x 3 around the centres
    avg = O.psf_average([a, b], max_size=False)
    assert avg.shape == (3, 3, 1) and avg[1, 1, 0] == np.float32(7)
    # make the same size: centred, extended with the minimum
    s = O.psf_make_same_size(a + 5, (5, 3, 5))
    assert s.shape == (5, 3, 5) and s[0, 0, 0] == 5 and s[2, 1, 2] == 5 + 13
    # projections: max along the smallest axis (x for b: size 1), min along y
    pr, d = O.psf_projection(b, -1, True)
    assert d == 0 and pr.shape == (5, 3) and np.all(pr == 1)
    pr, d = O.psf_projection(a, 1, False)
    assert d == 1 and pr.shape == (3, 3) and np.array_equal(pr, a[:, 0, :])
    # removing the min projections of a separable ramp leaves zeros
    r = (np.arange(4)[None, None, :] + 10 * np.arange(3)[None, :, None] + 100 * np.arange(5)[:, None, None])
    assert not O.psf_remove_min_projections(r.astype(np.float32)).any()


def test_nlinear_against_direct_trilinear():
    # the Gray-code float accumulation of the corners agrees with the exact trilinear form to
    # float rounding, and reproduces the corner values at integer positions exactly
    rng = np.random.default_rng(2)
    img = rng.uniform(0, 100, (6, 7, 8)).astype(np.float32)
    t = rng.uniform(0, 1, (200, 3)) * np.array([6.99, 5.99, 4.99])

    def get(ix, iy, iz):
        return img[iz, iy, ix]

    got = O.nlinear(get, t).astype(np.float64)
    f = np.floor(t).astype(int)
    w = t - f
    ref = np.zeros(len(t))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                c = ((w[:, 0] if dx else 1 - w[:, 0]) * (w[:, 1] if dy else 1 - w[:, 1]) *
                     (w[:, 2] if dz else 1 - w[:, 2]))
                ref += c * img[f[:, 2] + dz, f[:, 1] + dy, f[:, 0] + dx]
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    ti = np.array([[3, 2, 1], [0, 0, 0], [6, 5, 4]], dtype=np.float64)
    assert np.array_equal(O.nlinear(get, ti), img[[1, 0, 4], [2, 0, 5], [3, 0, 6]])


def test_psf_projection_and_average_edge_cases():
    # projections skip NaN (the comparison fails) and an all-NaN line keeps the start value;
    # the smallest-size average of equal sizes is the plain mean
    a = np.ones((3, 4, 5), np.float32)
    a[1, 2, 3] = np.nan
    a[:, 0, 0] = np.nan
    pr, d = O.psf_projection(a, 2, True)
    assert d == 2 and pr[2, 3] == 1 and pr[0, 0] == np.float32(-np.inf)
    b = np.full((3, 4, 5), 3, np.float32)
    assert np.array_equal(O.psf_average([np.ones_like(b), b], max_size=False), np.full_like(b, 2))


def test_psf_extract_against_scalar_loops():
    # the vectorised restatement of extractPSFLocal against its loops written out, element by
    # element, on a tiny periodic image
    import math

    rng = np.random.default_rng(4)
    img = rng.uniform(0, 10, (4, 5, 6)).astype(np.float32)  # [z][y][x]
    D = (6, 5, 4)
    size = (3, 5, 3)
    locs = [(0.25, 4.5, 3.75), (5.9, 0.1, 1.5)]
    ref = np.zeros((size[2], size[1], size[0]), np.float32)
    order = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, 1)]
    for l in locs:
        for z in range(size[2]):
            for y in range(size[1]):
                for x in range(size[0]):
                    t = [float(x - size[0] // 2) + l[0], float(y - size[1] // 2) + l[1], float(z - size[2] // 2) + l[2]]
                    f = [math.floor(v) for v in t]
                    w = [t[d] - f[d] for d in range(3)]
                    acc = None
                    for dx, dy, dz in order:
                        wt = ((w[0] if dx else 1 - w[0]) * (w[1] if dy else 1 - w[1])) * (w[2] if dz else 1 - w[2])
                        v = float(img[(f[2] + dz) % D[2], (f[1] + dy) % D[1], (f[0] + dx) % D[0]])
                        term = np.float32(v * wt)
                        acc = term if acc is None else np.float32(acc + term)
                    ref[z, y, x] = np.float32(float(ref[z, y, x]) + float(acc))
    assert np.array_equal(O.psf_extract(img, locs, size), ref)


def test_load_group_transform_psfs_same_size():
    rng = np.random.default_rng(6)
    p = rng.gamma(2.0, 1.0, (9, 7, 7)).astype(np.float32)
    ident = np.hstack([np.eye(3), np.zeros((3, 1))])
    rot = np.array([[0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]], dtype=np.float64)  # 90 degrees about y
    out = O.load_group_transform_psfs([[(p, ident)], [(p, rot)]], same_size_for_all=True)
    assert out[0].shape == out[1].shape == (9, 7, 9)
    # the identity group is the normalised PSF centred in the larger box, extended with its minimum (0)
    assert np.array_equal(out[0][:, :, 1:8], O.psf_normalize(p)) and not out[0][:, :, 0].any()
    sep = O.load_group_transform_psfs([[(p, ident)], [(p, rot)]], same_size_for_all=False)
    assert sep[0].shape == (9, 7, 7) and sep[1].shape == (7, 7, 9)
