"""Oracle (CPU) checks of the CEOS raw-data reader restatement and the test
writer: the 4-bit decode table, the AGC code, multi-block round trips with
the replica spliced into each block, and the reference's own RADARSAT-1
samples and attenuation codes."""
import os

import numpy as np

from oracle import ceos

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_decode_table():
    # 4-bit two's complement, 2 v + 1 (read_CEOS_raw.m:135-141)
    assert list(ceos.decode_nibble(np.arange(16))) == [1, 3, 5, 7, 9, 11, 13, 15, -15, -13, -11, -9, -7, -5, -3, -1]
    assert np.array_equal(ceos.decode_nibble(ceos.encode_nibble(np.arange(-15, 16, 2))), np.arange(-15, 16, 2))


def test_agc_code():
    assert list(ceos.agc_db([0, 12, 31, 32, 45, 63, 64 + 12])) == [0, 12, 31, 8, 21, 39, 12]


def test_round_trip_across_blocks():
    rng = np.random.default_rng(4)
    lay = ceos.CeosLayout()
    n, m = 37, 300
    v = (2 * rng.integers(-8, 8, (n, m)) + 1) + 1j * (2 * rng.integers(-8, 8, (n, m)) + 1)
    codes = rng.integers(0, 64, n)
    raw = ceos.write(v, codes, lay, first_cell=4000, seed=2)
    assert raw.size == lay.file_header + 5 * lay.block_bytes
    for first, cnt in ((0, 37), (5, 20), (13, 3), (31, 6)):
        e, a = ceos.read(raw, lay, first, cnt, 4000, m, apply_agc=False)
        assert np.array_equal(e, v[first:first + cnt].astype(np.complex64))
        assert np.array_equal(a, ceos.agc_db(codes[first:first + cnt]))


def test_reference_samples_and_attenuation():
    """The reference's extracted samples (CDdata*.mat, via the omega-K golden
    crop) and attenuation codes survive the writer and the reader; with the
    AGC the lines scale by 1.5 10^(dB/20) (load_DATA_block.m:58-69)."""
    crop = np.load(os.path.join(GOLD, "wk_cd_crop.npz"))["echo"]
    agc = np.load(os.path.join(GOLD, "ceos_agc.npz"))["agc_db"]
    lay = ceos.CeosLayout()
    raw = ceos.write(crop, agc, lay, first_cell=1049 + 1000, seed=3)
    e, a = ceos.read(raw, lay, 0, 96, 1049 + 1000, 64, apply_agc=False)
    assert np.array_equal(e, crop) and np.array_equal(a, agc)
    g, _ = ceos.read(raw, lay, 0, 96, 1049 + 1000, 64, apply_agc=True)
    assert np.allclose(g, crop * (1.5 * 10.0 ** (agc[:, None] / 20.0)), rtol=1e-6)
