"""TIFF-stack output (Save3dTIFF): layout, ImageJ description and a write/read round trip."""
import struct
import zipfile

import numpy as np

from spim_registration_gb300.export import Save3dTIFF, read_tiff_stack, tiff_bytes


def test_round_trip_and_header(tmp_path):
    rng = np.random.default_rng(1)
    img = (rng.random((5, 7, 9)) * 1000).astype(np.float32)
    b = tiff_bytes(img)
    assert b[:4] == b"MM\x00\x2a"  # big-endian TIFF, as ImageJ writes
    got, desc = read_tiff_stack(b)
    np.testing.assert_array_equal(got, img)
    assert "images=5" in desc and "slices=5" in desc and desc.startswith("ImageJ=")
    # one image file directory per slice, each with 32-bit float samples (SampleFormat 3)
    off = struct.unpack(">I", b[4:8])[0]
    n_ifd = 0
    while off:
        n = struct.unpack(">H", b[off:off + 2])[0]
        tags = {struct.unpack(">H", b[off + 2 + 12 * i:off + 4 + 12 * i])[0] for i in range(n)}
        assert {256, 257, 258, 273, 279, 339} <= tags
        off = struct.unpack(">I", b[off + 2 + 12 * n:off + 6 + 12 * n])[0]
        n_ifd += 1
    assert n_ifd == 5


def test_save3dtiff_calibration_and_zip(tmp_path):
    img = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4)
    Save3dTIFF(str(tmp_path)).exportImage(img, "fused", bb_min_xyz=(10, -4, 6), downsampling=2.0, min_max=(0, 50))
    got, desc = read_tiff_stack(str(tmp_path / "fused.tif"))
    np.testing.assert_array_equal(got, img)
    assert "xorigin=-5.0" in desc and "yorigin=2.0" in desc and "zorigin=-3.0" in desc
    assert "spacing=2.0" in desc and "min=0.0" in desc and "max=50.0" in desc
    Save3dTIFF(str(tmp_path), compress=True).exportImage(img, "fusedz")
    with zipfile.ZipFile(tmp_path / "fusedz.zip") as z:
        got2, _ = read_tiff_stack(z.read("fusedz.tif"))
    np.testing.assert_array_equal(got2, img)
