"""Export of the deconvolved volume through the C ABI (host buffers: file formats only, no GPU
work, so these run without a GPU):

* mvr_export_tiff: an ImageJ stack of 32-bit float slices (Save3dTIFF.saveTiffStack), read back
  with a TIFF reader written here from the TIFF 6.0 layout: every slice, the ImageJ description
  (slice count, unit, z spacing, display range 0..255) and the x / y resolution;
* mvr_export_n5: an N5 float32 dataset of raw blocks (ExportN5Api), every block file read back
  (header: mode, number of dimensions, block size; big-endian values).

Both bit-exact (float values are copied, only their byte order changes).
"""
import json
import os
import struct

import numpy as np
import pytest

import mvrgb300 as M


def read_tiff(path):
    """The slices and the tags of the first IFD of a big-endian TIFF stack."""
    data = open(path, "rb").read()
    assert data[:4] == b"MM\x00\x2a"
    off = struct.unpack(">I", data[4:8])[0]
    slices, first = [], None
    while off:
        n = struct.unpack(">H", data[off:off + 2])[0]
        tags = {}
        for i in range(n):
            tid, typ, cnt = struct.unpack(">HHI", data[off + 2 + 12 * i:off + 10 + 12 * i])
            raw = data[off + 10 + 12 * i:off + 14 + 12 * i]
            tags[tid] = (typ, cnt, struct.unpack(">H", raw[:2])[0] if typ == 3 else struct.unpack(">I", raw)[0])
        if first is None:
            first = tags
        w, h = tags[256][2], tags[257][2]
        assert tags[258][2] == 32 and tags[339][2] == 3 and tags[259][2] == 1
        so, sc = tags[273][2], tags[279][2]
        assert sc == 4 * w * h
        slices.append(np.frombuffer(data[so:so + sc], dtype=">f4").reshape(h, w))
        off = struct.unpack(">I", data[off + 2 + 12 * n:off + 6 + 12 * n])[0]
    typ, cnt, doff = first[270]
    desc = data[doff:doff + cnt - 1].decode()
    xr = struct.unpack(">II", data[first[282][2]:first[282][2] + 8])
    return np.stack(slices), desc, xr


def test_tiff_stack_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    vol = rng.normal(100, 30, (7, 20, 33)).astype(np.float32)  # [z][y][x]
    vol[0, 0, 0] = -0.0
    vol[1, 2, 3] = np.float32(1e-38)
    p = tmp_path / "psi.tif"
    M.export_tiff(p, vol, calibration=(0.5, 0.5, 2.0), unit="um")
    got, desc, xr = read_tiff(p)
    assert got.shape == vol.shape
    assert np.array_equal(got.astype(np.float32).view(np.uint32), vol.view(np.uint32))
    lines = dict(l.split("=", 1) for l in desc.strip().split("\n"))
    assert lines["images"] == "7" and lines["slices"] == "7" and lines["unit"] == "um"
    assert float(lines["spacing"]) == 2.0 and float(lines["min"]) == 0.0 and float(lines["max"]) == 255.0
    assert xr[0] / xr[1] == pytest.approx(2.0)  # pixels per unit = 1 / 0.5


def test_n5_raw_blocks_round_trip(tmp_path):
    rng = np.random.default_rng(4)
    vol = rng.uniform(0, 1, (21, 18, 30)).astype(np.float32)
    M.export_n5(tmp_path / "out.n5", "psi", vol, block_size=(16, 8, 10))
    attrs = json.load(open(tmp_path / "out.n5" / "psi" / "attributes.json"))
    assert attrs["dimensions"] == [30, 18, 21] and attrs["blockSize"] == [16, 8, 10]
    assert attrs["dataType"] == "float32" and attrs["compression"] == {"type": "raw"}
    back = np.full(vol.shape, np.nan, np.float32)
    for bx in range(2):
        for by in range(3):
            for bz in range(3):
                raw = open(tmp_path / "out.n5" / "psi" / str(bx) / str(by) / str(bz), "rb").read()
                mode, nd = struct.unpack(">HH", raw[:4])
                nx, ny, nz = struct.unpack(">III", raw[4:16])
                assert mode == 0 and nd == 3
                assert (nx, ny, nz) == (min(16, 30 - 16 * bx), min(8, 18 - 8 * by), min(10, 21 - 10 * bz))
                blk = np.frombuffer(raw[16:], dtype=">f4").reshape(nz, ny, nx)
                back[10 * bz:10 * bz + nz, 8 * by:8 * by + ny, 16 * bx:16 * bx + nx] = blk
    assert np.array_equal(back, vol)


def test_export_errors(tmp_path):
    vol = np.zeros((2, 3, 4), np.float32)
    with pytest.raises(M.MvrError) as e:
        M.export_tiff(tmp_path / "missing_dir" / "x.tif", vol)
    assert "cannot open" in str(e.value)
    with pytest.raises(M.MvrError):
        M.export_n5(tmp_path / "o.n5", "d", vol, block_size=(0, 1, 1))
    assert not os.path.exists(tmp_path / "missing_dir")


@pytest.mark.gpu
def test_export_from_device_memory(tmp_path):
    # psi as the whole-volume driver leaves it on the device (read back in slabs)
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    vol = rng.uniform(0, 5, (9, 31, 17)).astype(np.float32)
    d = torch.from_numpy(vol).cuda()
    M.export_tiff(tmp_path / "d.tif", d.data_ptr(), dims=(17, 31, 9))
    got, _, _ = read_tiff(tmp_path / "d.tif")
    assert np.array_equal(got.astype(np.float32), vol)
    M.export_n5(tmp_path / "d.n5", "psi", d.data_ptr(), block_size=(8, 16, 4), dims=(17, 31, 9))
    raw = open(tmp_path / "d.n5" / "psi" / "2" / "1" / "2", "rb").read()
    nx, ny, nz = struct.unpack(">III", raw[4:16])
    assert (nx, ny, nz) == (1, 15, 1)
    assert np.array_equal(np.frombuffer(raw[16:], dtype=">f4").reshape(nz, ny, nx), vol[8:9, 16:31, 16:17])
