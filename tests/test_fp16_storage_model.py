"""FP16 storage of range-compressed rows: the scale rule and its error, on the CPU.

The FP16-storage mode keeps each pulse's upsampled, range-compressed row as
complex half precision with a per-pulse power-of-two scale (csrc/rc.cu): the
forward transform sums |Y[k]| over the matched-filtered spectrum, a bound on
every output of the inverse, and the scale 2^ceil(log2(bound) - 14) keeps the
stored magnitudes within 2^14 (half precision overflows past 65504); the rows
are stored rounded to nearest, as numpy's float16 rounds.  Restated here on the
oracle's own rows (FP64 range compression of the configured scenes' echoes,
BPA_SAR.m:93-111 restated in oracle/):
  * no stored value exceeds 2^14, at every configured FFT size;
  * the stored rows are within -71 to -76 dB relative L2 of the exact ones:
    half precision's rounding (a 10-bit fraction), which is what limits the
    FP16-storage images (config 2 on the GPU: -73.7 dB against the oracle,
    the same figure), not the split arithmetic.
"""
import math

import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import scenes


def stored_rows(s):
    from oracle import oracle as orc
    r, lay = s.radar, s.layout
    e = orc.echo(s).astype(np.complex64).astype(np.complex128)  # the GPU's complex64 input
    rows = orc.range_compress(s, e)
    # the forward transform's bound: sum_k |FFT_N(echo)[k] filt[k]|, filt the matched
    # filter with the output lag shift and 1/N
    h = orc.chirp(lay.nc, 1.0 / r.fs, r.kr, r.tp, r.tp / 2.0, False)
    H = np.fft.fft(np.concatenate([h, np.zeros(lay.nfft - lay.nc)]))
    k = np.arange(lay.nfft)
    filt = np.conj(H) * np.exp(-2j * np.pi * ((k * lay.shift) % lay.nfft) / lay.nfft) / lay.nfft
    E = np.fft.fft(np.concatenate([e, np.zeros((s.np_, lay.nfft - s.ns))], axis=1), axis=1)
    bound = np.sum(np.abs(E * filt), axis=1)
    scale = 2.0 ** np.ceil(np.log2(bound) - 14.0)
    x = rows / scale[:, None]
    half = x.real.astype(np.float16).astype(np.float64) + 1j * x.imag.astype(np.float16).astype(np.float64)
    return rows, x, half * scale[:, None], bound / scale


@pytest.mark.parametrize("name,make", [("config1", lambda: scenes.config1(np_=32)),
                                       ("config2", lambda: scenes.config2(np_=16, n_img=256)),
                                       ("config5", lambda: scenes.config5(np_=8, n_img=256))])
def test_fp16_rows(name, make):
    s = make()
    rows, x, stored, scaled_bound = stored_rows(s)
    peak = np.max(np.abs(x), axis=1)
    assert np.all(scaled_bound <= 2.0 ** 14) and np.all(peak <= scaled_bound), name  # the bound covers every output
    assert np.all(np.isfinite(stored)), name
    err = 20.0 * math.log10(np.linalg.norm(stored - rows) / np.linalg.norm(rows))
    print(name, f"FP16 rows {err:.1f} dB, largest stored magnitude {peak.max():.0f}")
    assert -76.0 <= err <= -71.0, (name, err)
