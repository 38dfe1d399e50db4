"""Synthetic stripmap scenes: radar constants, antenna phase-centre tracks,
pixel grids and point-target lists for the imaging workloads.

The radar constants replace the compile-time ``SARParams`` defaults of the
reference (code/SAR_BP/CUDA/BPA_CUDA.h:28-50) and the parameter block of its
MATLAB specification (code/SAR_BP/matlab/BPA_SAR.m:7-51).  Unlike the
reference, the APC track and the pixel grid are explicit arrays/structs.

Geometry (slant plane, APC altitude 0):
  world X = along-track (azimuth), world Y = cross-track range, world Z = up.
  APC_p = (V * (p - (Np-1)/2) / PRF, 0, 0) plus optional motion error.
  Image rows run along azimuth and columns along range, as in the reference's
  ``idx = i*Nr + j`` (BPA_CUDA_kernels.cu:49-53): ux = (0, d, 0) steps one column
  in range, uy = (d, 0, 0) steps one row in azimuth, and the scene centre
  (0, R0, 0) sits on pixel (Nx/2, Ny/2).

Signal conventions (shared by the oracle and the CUDA path):
  * LFM chirp centred at baseband, exp(j*pi*Kr*(u - Tp/2)^2) for u in [0, Tp).
    BPA_SAR.m uses an uncentred chirp (band [0, B]); with fs = 1.2 B that band
    would alias, so the chirp is centred.
  * Echo sample n has delay t_rec0 + n/fs; the record is centred on the
    scene-centre echo: t_rec0 = 2 R0/c + Tp/2 - Ns/(2 fs).
  * Range compression is a linear correlation (N_fft = nextpow2(Ns + Nc - 1)),
    output lag shifted by D = Nc // 2 so compressed sample i has delay
    t_rec0 + (i - D)/fs; upsampled bin b has delay t0_bins + b/(L fs) with
    t0_bins = t_rec0 - D/fs.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

C_LIGHT = 3.0e8  # the reference's value (BPA_CUDA.h:29, BPA_SAR.m:7)


@dataclasses.dataclass
class Radar:
    c: float = C_LIGHT
    fc: float = 5.3e9
    bandwidth: float = 100e6
    tp: float = 10e-6
    fs: float = 120e6
    prf: float = 500.0
    v: float = 150.0
    r0: float = 5000.0
    upsample: int = 8

    @property
    def kr(self) -> float:
        return self.bandwidth / self.tp

    @property
    def wavelength(self) -> float:
        return self.c / self.fc


@dataclasses.dataclass
class Grid:
    origin: np.ndarray  # (3,) float64, position of pixel (0, 0)
    ux: np.ndarray      # (3,) step of one column (x index)
    uy: np.ndarray      # (3,) step of one row (y index)
    nx: int
    ny: int

    def pixel(self, x, y):
        return self.origin + np.multiply.outer(x, self.ux) + np.multiply.outer(y, self.uy)


@dataclasses.dataclass
class RcLayout:
    nc: int          # chirp samples round(Tp*fs)
    nfft: int        # nextpow2(Ns + Nc - 1)
    shift: int       # lag shift D = Nc // 2
    nbins: int       # L * Ns upsampled bins per pulse
    t0_bins: float   # delay of upsampled bin 0
    bin_rate: float  # L * fs


def next_pow2(n: int) -> int:
    return 1 << max(0, int(n - 1).bit_length())


def rc_layout(radar: Radar, ns: int, t_rec0: float) -> RcLayout:
    nc = int(round(radar.tp * radar.fs))
    nfft = next_pow2(ns + nc - 1)
    shift = nc // 2
    return RcLayout(nc=nc, nfft=nfft, shift=shift, nbins=radar.upsample * ns,
                    t0_bins=t_rec0 - shift / radar.fs,
                    bin_rate=radar.upsample * radar.fs)


@dataclasses.dataclass
class Scene:
    name: str
    radar: Radar
    np_: int                 # pulses
    ns: int                  # range samples per pulse
    apc: np.ndarray          # (np, 3) float64
    grid: Grid
    targets: np.ndarray      # (nt, 4) float64: x, y, z, amplitude
    t_rec0: float
    snr_db: float | None
    seed: int

    @property
    def layout(self) -> RcLayout:
        return rc_layout(self.radar, self.ns, self.t_rec0)

    @property
    def updates(self) -> int:
        return self.grid.nx * self.grid.ny * self.np_


def straight_track(radar: Radar, n_pulses: int) -> np.ndarray:
    t = (np.arange(n_pulses, dtype=np.float64) - (n_pulses - 1) / 2.0) / radar.prf
    apc = np.zeros((n_pulses, 3), dtype=np.float64)
    apc[:, 0] = radar.v * t
    return apc


def curved_track(radar: Radar, n_pulses: int, amp: float = 0.5, period: float = 200.0,
                 jitter: float = 0.02, seed: int = 5) -> np.ndarray:
    """Straight track plus sinusoidal cross-track error and Gaussian jitter."""
    apc = straight_track(radar, n_pulses)
    rng = np.random.default_rng(seed)
    apc[:, 1] += amp * np.sin(2.0 * math.pi * apc[:, 0] / period)
    apc[:, 1] += rng.normal(0.0, jitter, n_pulses)
    apc[:, 2] += rng.normal(0.0, jitter, n_pulses)
    return apc


def centred_grid(radar: Radar, nx: int, ny: int, spacing: float) -> Grid:
    ux = np.array([0.0, spacing, 0.0])
    uy = np.array([spacing, 0.0, 0.0])
    centre = np.array([0.0, radar.r0, 0.0])
    origin = centre - (nx // 2) * ux - (ny // 2) * uy
    return Grid(origin=origin, ux=ux, uy=uy, nx=nx, ny=ny)


def centred_record_start(radar: Radar, ns: int) -> float:
    return 2.0 * radar.r0 / radar.c + radar.tp / 2.0 - ns / (2.0 * radar.fs)


def grid_targets_3x3(radar: Radar, spacing: float = 20.0) -> np.ndarray:
    t = []
    for da in (-spacing, 0.0, spacing):
        for dr in (-spacing, 0.0, spacing):
            t.append((da, radar.r0 + dr, 0.0, 1.0))
    return np.array(t, dtype=np.float64)


def random_targets(grid: Grid, n: int, seed: int, margin: float = 0.05) -> np.ndarray:
    """Uniform positions over the imaged area, Rayleigh(sigma=1) amplitudes."""
    rng = np.random.default_rng(seed)
    fx = rng.uniform(margin, 1.0 - margin, n) * grid.nx
    fy = rng.uniform(margin, 1.0 - margin, n) * grid.ny
    pos = grid.origin + np.outer(fx, grid.ux) + np.outer(fy, grid.uy)
    amp = rng.rayleigh(1.0, n)
    return np.column_stack([pos, amp]).astype(np.float64)


def isolated_targets(grid: Grid, seed: int,
                     fractions=((0.22, 0.26), (0.71, 0.21), (0.48, 0.52), (0.24, 0.77), (0.79, 0.74))) -> np.ndarray:
    """Point targets far enough apart for point-target metrics (image
    fractions of the grid, default five), each moved by a random sub-pixel
    offset, with Rayleigh(sigma=1) amplitudes kept above 0.5."""
    rng = np.random.default_rng(seed)
    out = []
    for fx, fy in fractions:
        x = fx * grid.nx + rng.uniform(-0.5, 0.5)
        y = fy * grid.ny + rng.uniform(-0.5, 0.5)
        pos = grid.origin + x * grid.ux + y * grid.uy
        out.append((*pos, max(0.5, rng.rayleigh(1.0))))
    return np.array(out, dtype=np.float64)


def config1(np_: int = 512, ns: int = 1024, n_img: int = 512, spacing: float = 0.5,
            seed: int = 1, snr_db: float | None = 30.0) -> Scene:
    """Plain BP point-target scene: 512 pulses x 1024 samples, 3x3 targets
    spaced 20 m, 30 dB SNR, 512^2 image at 0.5 m."""
    radar = Radar()
    return Scene(name="c1", radar=radar, np_=np_, ns=ns, apc=straight_track(radar, np_),
                 grid=centred_grid(radar, n_img, n_img, spacing),
                 targets=grid_targets_3x3(radar), t_rec0=centred_record_start(radar, ns),
                 snr_db=snr_db, seed=seed)


def config2(np_: int = 4096, ns: int = 8192, n_img: int = 4096, spacing: float = 0.25,
            n_targets: int = 200, seed: int = 2, snr_db: float | None = 20.0) -> Scene:
    """Larger scene: 4096 pulses x 8192 samples, 200 Rayleigh targets uniform
    over the image, 20 dB clutter, 4096^2 image at 0.25 m."""
    radar = Radar()
    grid = centred_grid(radar, n_img, n_img, spacing)
    return Scene(name="c2", radar=radar, np_=np_, ns=ns, apc=straight_track(radar, np_),
                 grid=grid, targets=random_targets(grid, n_targets, seed),
                 t_rec0=centred_record_start(radar, ns), snr_db=snr_db, seed=seed)


def config5(np_: int = 16384, ns: int = 16384, n_img: int = 8192, spacing: float = 0.25,
            n_targets: int = 200, seed: int = 5, snr_db: float | None = 20.0) -> Scene:
    """Large curved-track stripmap: 16384 x 16384 echo, 0.5 m / 200 m sinusoidal
    cross-track error + 2 cm jitter, 8192^2 image."""
    radar = Radar()
    grid = centred_grid(radar, n_img, n_img, spacing)
    return Scene(name="c5", radar=radar, np_=np_, ns=ns, apc=curved_track(radar, np_, seed=seed),
                 grid=grid, targets=random_targets(grid, n_targets, seed),
                 t_rec0=centred_record_start(radar, ns), snr_db=snr_db, seed=seed)


def noise_sigma(clean_mean_power: float, snr_db: float) -> float:
    """Noise standard deviation (complex, total) for a given SNR relative to the
    mean noiseless echo power."""
    return math.sqrt(clean_mean_power / (10.0 ** (snr_db / 10.0)))


def ground_scene(np_: int = 256, ns: int = 2048, n_img: int = 256, spacing: float = 1.0, altitude: float = 5000.0,
                 ground_range: float = 10000.0, seed: int = 7, snr_db: float | None = 30.0) -> Scene:
    """Airborne geometry with the image on the ground (the reference program's
    data model: antenna at altitude H, pixels at z = 0, 1 m spacing,
    BPA_CUDA.cpp:26-48), 3x3 targets around the scene centre."""
    radar = Radar()
    apc = straight_track(radar, np_)
    apc[:, 2] = altitude
    ux = np.array([0.0, spacing, 0.0])
    uy = np.array([spacing, 0.0, 0.0])
    centre = np.array([0.0, ground_range, 0.0])
    grid = Grid(origin=centre - (n_img // 2) * ux - (n_img // 2) * uy, ux=ux, uy=uy, nx=n_img, ny=n_img)
    r0 = float(np.hypot(ground_range, altitude))
    t = []
    for da in (-20.0, 0.0, 20.0):
        for dr in (-20.0, 0.0, 20.0):
            t.append((da, ground_range + dr, 0.0, 1.0))
    t_rec0 = 2.0 * r0 / radar.c + radar.tp / 2.0 - ns / (2.0 * radar.fs)
    return Scene(name="ground", radar=radar, np_=np_, ns=ns, apc=apc, grid=grid, targets=np.array(t),
                 t_rec0=t_rec0, snr_db=snr_db, seed=seed)
