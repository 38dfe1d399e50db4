"""Host-side tables and launch rules of the library, checked on the CPU.

A g++ harness calls the library's own host code (plan.cpp) and writes what it
builds; numpy restates each from its definition:
  * the matched-filter spectrum of range compression, conj(FFT_N(h)) times
    the output lag shift e^{-j 2 pi k shift / N} and 1/N, with h the reference
    chirp exp(j pi Kr (t - tc)^2) over the pulse (BPA_SAR.m:93-100; the
    oracle's own chirp), and the two-level phase table E^m = e^{+j 2 pi m /
    (L N)} of the upsampling inverse, at the configured layouts: FP32 values
    within 2^-23 of their magnitude;
  * the Bluestein tables of the omega-K row DFT (w_j = e^{j pi j^2 / n}, the
    m-point transforms of the circular kernel and of its conjugate, / m), used
    through the Bluestein identity in numpy: a DFT of length n within 1e-6 of
    numpy's at lengths that are not powers of two;
  * the back-projection's pulse-segment rule over a sweep of launches: the
    fewest segments that give at least 12 waves of 2 CTAs per SM, at least 4
    chunks of 16 pulses per segment, no empty segment, partial images within
    1 GiB, and a forced count taken as given.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sar_cambrianaccelerationcard_gb300")
LIB = os.path.join(PKG, "libsarbp.so")

HARNESS = r"""
#include <cstdio>
#include <cstring>
#include <vector>
#include "sarbp_internal.h"
static void put(const std::vector<float2> &v) {
    const int n = (int)v.size();
    fwrite(&n, 4, 1, stdout);
    fwrite(v.data(), sizeof(float2), v.size(), stdout);
}
int main(int argc, char **argv) {
    if (argc < 2) return 2;
    if (!strcmp(argv[1], "rc")) {  // stdin: c fc fs kr tp tc t_rec0 (f64), upsample ns (i32)
        double d[7];
        int iv[2];
        if (fread(d, 8, 7, stdin) != 7 || fread(iv, 4, 2, stdin) != 2) return 1;
        sarbp_radar r{};
        r.c = d[0]; r.fc = d[1]; r.fs = d[2]; r.kr = d[3]; r.tp = d[4]; r.tc = d[5]; r.t_rec0 = d[6];
        r.upsample = iv[0];
        sarbp_rc_layout lay;
        if (sarbp_rc_layout_get(&r, iv[1], &lay) != SARBP_OK) return 3;
        std::vector<float2> filt, etab;
        sarbp::rc_tables_host(r, lay, filt, etab);
        const int hdr[3] = {lay.nc, lay.nfft, lay.shift};
        fwrite(hdr, 4, 3, stdout);
        put(filt);
        put(etab);
        return 0;
    }
    if (!strcmp(argv[1], "dft")) {  // argv[2] = n
        const int n = atoi(argv[2]);
        std::vector<float2> etab, chirp, kf, ki;
        sarbp::dft_tables_host(n, etab, chirp, kf, ki);
        const int m = sarbp::dft_bluestein_size(n);
        fwrite(&m, 4, 1, stdout);
        put(chirp);
        put(kf);
        put(ki);
        return 0;
    }
    if (!strcmp(argv[1], "seg")) {  // stdin lines: tiles npl npix sms force
        int tiles, npl, sms, force;
        long long npix;
        printf("%d\n", sarbp::bp_max_chunk());
        while (scanf("%d %d %lld %d %d", &tiles, &npl, &npix, &sms, &force) == 5)
            printf("%d\n", sarbp::bp_choose_segments(tiles, npl, npix, sms, force));
        return 0;
    }
    return 2;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    inc = None
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            inc = os.path.join(d, "include")
            break
    if not (shutil.which("g++") and inc and os.path.exists(LIB)):
        pytest.skip("needs g++, the CUDA headers and the built library")
    d = tmp_path_factory.mktemp("tables")
    src, exe = d / "harness.cpp", d / "harness"
    src.write_text(HARNESS)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "csrc"),
                    "-I", inc, str(src), "-o", str(exe), LIB, f"-Wl,-rpath,{PKG}"], check=True)

    def run(args, data=b"", text=False):
        out = subprocess.run([str(exe)] + args, input=data, capture_output=True, check=True)
        return out.stdout.decode() if text else out.stdout

    return run


def take(buf, off):
    n = struct.unpack_from("i", buf, off)[0]
    v = np.frombuffer(buf, dtype=np.float32, count=2 * n, offset=off + 4)
    return v[0::2].astype(np.float64) + 1j * v[1::2].astype(np.float64), off + 4 + 8 * n


def close(got, ref, rel):
    return float(np.max(np.abs(got - ref))) <= rel * float(np.max(np.abs(ref)))


@pytest.mark.parametrize("name,ns,upsample", [("config1", 1024, 8), ("config2", 8192, 8), ("config5", 16384, 8),
                                              ("ragged", 3001, 4), ("short", 100, 16)])
def test_range_compression_tables(harness, name, ns, upsample):
    from oracle import oracle as orc
    r = scenes.Radar()
    r.upsample = upsample
    t_rec0 = 3.3e-5
    data = struct.pack("7d", r.c, r.fc, r.fs, r.kr, r.tp, r.tp / 2.0, t_rec0) + struct.pack("2i", upsample, ns)
    buf = harness(["rc"], data)
    nc, nfft, shift = struct.unpack_from("3i", buf, 0)
    lay = scenes.rc_layout(r, ns, t_rec0)
    assert (nc, nfft, shift) == (lay.nc, lay.nfft, lay.shift)
    filt, off = take(buf, 12)
    etab, off = take(buf, off)
    assert off == len(buf) and filt.size == nfft
    h = orc.chirp(nc, 1.0 / r.fs, r.kr, r.tp, r.tp / 2.0, False)
    H = np.fft.fft(np.concatenate([h, np.zeros(nfft - nc)]))
    k = np.arange(nfft)
    ref = np.conj(H) * np.exp(-2j * np.pi * ((k * shift) % nfft) / nfft) / nfft
    assert close(filt, ref, 2.0 ** -23), name
    LN = upsample * nfft
    m = np.concatenate([np.arange(256), 256 * np.arange(etab.size - 256)])
    assert etab.size == 256 + max(LN // 256, 1)
    assert close(etab, np.exp(2j * np.pi * m / LN), 2.0 ** -23), name


@pytest.mark.parametrize("n", [3, 100, 1000, 2500, 7919])
def test_bluestein_tables_give_the_dft(harness, n):
    buf = harness(["dft", str(n)])
    m = struct.unpack_from("i", buf, 0)[0]
    assert m >= 2 * n - 1 and m & (m - 1) == 0
    chirp, off = take(buf, 4)
    kf, off = take(buf, off)
    ki, off = take(buf, off)
    assert chirp.size == n and kf.size == m and ki.size == m
    j = np.arange(n)
    w = np.exp(1j * np.pi * ((j * j) % (2 * n)) / n)
    assert close(chirp, w, 2.0 ** -23)
    x = np.random.default_rng(n).standard_normal(n) + 1j * np.random.default_rng(n + 1).standard_normal(n)
    # X_k = conj(w_k) sum_j (x_j conj(w_j)) w_{k-j}: the convolution through m-point transforms
    a = np.zeros(m, complex)
    a[:n] = x * np.conj(chirp)
    fwd = np.conj(chirp) * (np.fft.ifft(np.fft.fft(a) * kf) * m)[:n]
    assert close(fwd, np.fft.fft(x), 1e-6), n
    # inverse: X_k = w_k sum_j (x_j w_j) conj(w_{k-j}), unnormalised
    a[:n] = x * chirp
    inv = chirp * (np.fft.ifft(np.fft.fft(a) * ki) * m)[:n]
    assert close(inv, np.fft.ifft(x) * n, 1e-6), n


def test_pulse_segment_rule(harness):
    sms = 152
    cases = []
    for tiles in (1, 7, 64, 152, 300, 1000, 2048, 8192, 16384):
        for npl in (1, 16, 63, 64, 100, 512, 1000, 4096, 16384):
            for npix in (512 * 512, 4096 * 4096, 8192 * 8192):
                cases.append((tiles, npl, npix, sms, 0))
    cases += [(100, 4096, 4096 * 4096, sms, f) for f in (1, 3, 64)]
    out = harness(["seg"], "".join(" ".join(map(str, c)) + "\n" for c in cases).encode(), text=True).split()
    kc = int(out[0])
    assert kc == 16
    seen = set()
    for (tiles, npl, npix, sm, force), s in zip(cases, map(int, out[1:])):
        if force:
            assert s == force
            continue
        target = 12 * 2 * sm

        def allowed(k):  # pulses and memory allow k segments (monotone in k)
            return k == 1 or (npl // k >= 4 * kc and k * npix * 8 <= 2 ** 30)

        def valid(k):  # ... and none of them is empty (pulses per segment in whole chunks)
            pps = -(-(-(-npl // k)) // kc) * kc
            return allowed(k) and (k == 1 or (k - 1) * pps < npl)

        assert 1 <= s <= 64 and valid(s), (tiles, npl, npix, s)
        # the fewest that reach the target ...
        assert not any(valid(k) and tiles * k >= target for k in range(1, s)), (tiles, npl, npix, s)
        # ... or, short of it, the most the pulses and memory allow
        if tiles * s < target:
            assert not any(valid(k) for k in range(s + 1, 65) if allowed(k)), (tiles, npl, npix, s)
        seen.add((s > 1, tiles * s >= target))
    assert seen == {(False, False), (False, True), (True, False), (True, True)}, seen
