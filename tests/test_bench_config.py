"""bench.py workload definitions (CPU): block grids of the three workloads follow the
reference's DeconView / BlockGeneratorFixedSizePrecise geometry (the doubled kernel 2k-1)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_workload_block_grids():
    w = bench.WORKLOADS["4view256"]()
    assert [len(w.blocks(v)) for v in range(4)] == [16] * 4  # 2 x 2 x 4 blocks of 192^3
    assert w.view_blocks_per_iter() == 64 and w.metric == "voxel-iterations/s (4 views)"
    w = bench.WORKLOADS["6view512fixed"]()
    # effective sizes 192 - 2(k-1): 152 ... 112 in x/y, 256 - 2(k-1): 176 ... 96 in z
    assert [len(w.blocks(v)) for v in range(6)] == [32, 32, 32, 32, 75, 75]
    # 128^3 effective blocks plus each view's overlap: 4 x 4 x 2 blocks in every view
    w = bench.WORKLOADS["6view512tight"]()
    assert w.per_view_blocks() and [len(w.blocks(v)) for v in range(6)] == [32] * 6
    for v, k in enumerate(w.psfs):
        b = w.vblocks[v]
        assert all(b[d] >= 128 + 2 * (k[d] - 1) for d in range(3))
        assert all(w.blocks(v)[0]["eff_size"][d] >= 128 for d in range(3))  # the last block may be clipped
    # the same effective grid with plane-kernel compute blocks: every block's effective
    # region where the reference's blocks (effective + 2 (k - 1)) put it, centred in a
    # compute block with at least k - 1 of overlap on each side
    w = bench.WORKLOADS["6view512"]()
    assert w.vblocks == [(192, 192, 256)] * 4 + [(256, 256, 288)] * 2 and w.effective == (128, 128, 128)
    for v, k in enumerate(w.psfs):
        g, r = w.blocks(v), w.ref_blocks(v)
        assert len(g) == 32 and w.ref_vblocks()[v] == tuple(128 + 2 * (k[d] - 1) for d in range(3))
        assert [(b["eff_offset"], b["eff_size"]) for b in g] == [(b["eff_offset"], b["eff_size"]) for b in r]
        for b in g:
            for d in range(3):
                lo = b["eff_offset"][d] - b["offset"][d]
                hi = w.vblocks[v][d] - lo - b["eff_size"][d]
                assert lo >= k[d] - 1 and hi >= k[d] - 1
    w = bench.WORKLOADS["8view1024"]()
    assert [len(w.blocks(v)) for v in range(8)] == [216] * 8


def test_workload_config_fields():
    for name, make in bench.WORKLOADS.items():
        w = make()
        c = w.config("circular")
        blk = [list(b) for b in w.vblocks] if w.per_view_blocks() else list(w.block)
        assert c["views"] == w.views and c["dims"] == list(w.dims) and c["block"] == blk
        assert ("inputs larger than L2" in c["l2"]) != w.flush_l2()
    assert bench.WORKLOADS["2view128"]().flush_l2() and not bench.WORKLOADS["4view256"]().flush_l2()


def test_reference_arm_line_on_the_two_view_workload():
    # the CPU arm end to end (float32 padded R2C restatement, one block per view per step)
    import json
    import subprocess

    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "2view128", "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "voxel-iterations/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # one step advances the whole 128x128x64 volume by one iteration (one block)
    assert abs(line["value"] * line["ms_per_step"] / 1e3 - 128 * 128 * 64) < 1.0
