"""CPU checks of the Rgba8p -> SRgba8 / Matte8 -> SGray8 table (the conversion pix
performs in footile's examples; restated from the sRGB standard, pix not vendored)."""
import numpy as np

import oracle


def test_srgb_table_known_values():
    t = oracle.srgb_table()
    # opaque row: the sRGB encoding of c / 255 (IEC 61966-2-1)
    assert list(t[255, [0, 1, 64, 128, 188, 255]]) == [0, 13, 137, 188, 223, 255]
    assert t[128, 64] == 188          # straight 0.5
    assert not t[0].any()             # alpha 0: no colour
    assert (t[10, 10:] == 255).all()  # channel >= alpha saturates
    assert (np.diff(t.astype(int), axis=1) >= 0).all()  # monotone in the channel


def test_convert_keeps_alpha_and_unpremultiplies():
    rng = np.random.default_rng(1)
    a = rng.integers(0, 256, (8, 9)).astype(np.uint8)
    rgb = (rng.random((8, 9, 3)) * a[..., None]).astype(np.uint8)
    src = np.concatenate([rgb, a[..., None]], axis=2)
    out = oracle.convert(src)
    assert np.array_equal(out[..., 3], a)
    full = np.full((4, 4, 4), 255, np.uint8)
    assert (oracle.convert(full) == 255).all()
    m = np.arange(256, dtype=np.uint8).reshape(16, 16)
    assert np.array_equal(oracle.convert(m), oracle.srgb_table()[255][m])
