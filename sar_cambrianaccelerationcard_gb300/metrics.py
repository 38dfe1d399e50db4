"""Image-quality metrics for back-projected images.

The reference assesses its images only visually: a -3 dB (0.707 * max)
contour of the magnitude (code/SAR_BP/matlab/BPA_SAR.m:168-175, :213-220).
These metrics make that quantitative and comparable between an image and the
FP64 oracle's image of the same scene:
  * relative L2 error in dB, 20 log10(||a - b|| / ||b||);
  * point-target peak position with sub-pixel accuracy (local FFT upsampling);
  * PSLR (peak side-lobe ratio) and ISLR (integrated side-lobe ratio) on the
    range and azimuth cuts through the peak;
  * -3 dB mainlobe widths (the reference's contour level) on both cuts.
"""
from __future__ import annotations

import dataclasses

import numpy as np


def rel_l2_db(a: np.ndarray, ref: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    num = np.linalg.norm((a - ref).ravel())
    den = np.linalg.norm(ref.ravel())
    if den == 0.0:
        return float("-inf") if num == 0.0 else float("inf")
    if num == 0.0:
        return float("-inf")
    return float(20.0 * np.log10(num / den))


@dataclasses.dataclass
class PointTarget:
    x: float          # sub-pixel peak column
    y: float          # sub-pixel peak row
    peak: float       # peak magnitude
    pslr_range_db: float
    pslr_azimuth_db: float
    islr_range_db: float
    islr_azimuth_db: float
    width_range: float    # -3 dB width, pixels
    width_azimuth: float  # -3 dB width, pixels


def _upsample_patch(patch: np.ndarray, up: int) -> np.ndarray:
    ny, nx = patch.shape
    F = np.fft.fftshift(np.fft.fft2(patch))
    big = np.zeros((ny * up, nx * up), dtype=np.complex128)
    y0 = (ny * up - ny) // 2
    x0 = (nx * up - nx) // 2
    big[y0:y0 + ny, x0:x0 + nx] = F
    return np.fft.ifft2(np.fft.ifftshift(big)) * (up * up)


def _cut_metrics(cut: np.ndarray, k: int, up: int):
    m = np.abs(cut)
    pk = m[k]
    left = k
    while left > 0 and m[left - 1] < m[left]:
        left -= 1
    right = k
    while right < len(m) - 1 and m[right + 1] < m[right]:
        right += 1
    side = np.concatenate([m[:left], m[right + 1:]])
    main = m[left:right + 1]
    pslr = 20.0 * np.log10(side.max() / pk) if side.size and side.max() > 0 else float("-inf")
    islr = 10.0 * np.log10((side ** 2).sum() / (main ** 2).sum()) if side.size else float("-inf")
    above = np.nonzero(m >= pk / np.sqrt(2.0))[0]
    # contiguous -3 dB region around the peak
    lo = k
    while lo - 1 in set(above) and lo - 1 >= 0:
        lo -= 1
    hi = k
    while hi + 1 < len(m) and m[hi + 1] >= pk / np.sqrt(2.0):
        hi += 1
    width = (hi - lo + 1) / up
    return pslr, islr, width


def point_target(img: np.ndarray, x_guess: int, y_guess: int, half: int = 16, up: int = 16) -> PointTarget:
    """Metrics of the point response nearest (x_guess, y_guess)."""
    img = np.asarray(img, dtype=np.complex128)
    ny, nx = img.shape
    # recentre on the brightest pixel of a small window
    y0, y1 = max(0, y_guess - 3), min(ny, y_guess + 4)
    x0, x1 = max(0, x_guess - 3), min(nx, x_guess + 4)
    w = np.abs(img[y0:y1, x0:x1])
    dy, dx = np.unravel_index(np.argmax(w), w.shape)
    yc, xc = y0 + dy, x0 + dx
    ya, yb = max(0, yc - half), min(ny, yc + half)
    xa, xb = max(0, xc - half), min(nx, xc + half)
    patch = img[ya:yb, xa:xb]
    U = _upsample_patch(patch, up)
    ky, kx = np.unravel_index(np.argmax(np.abs(U)), U.shape)
    pr, ir, wr = _cut_metrics(U[ky, :], kx, up)
    pa, ia, wa = _cut_metrics(U[:, kx], ky, up)
    return PointTarget(x=xa + kx / up, y=ya + ky / up, peak=float(np.abs(U[ky, kx])),
                       pslr_range_db=float(pr), pslr_azimuth_db=float(pa),
                       islr_range_db=float(ir), islr_azimuth_db=float(ia),
                       width_range=float(wr), width_azimuth=float(wa))


def compare_point_targets(img: np.ndarray, ref: np.ndarray, pixels) -> dict:
    """Largest differences over the listed target pixels (x, y) between img and ref."""
    out = {"peak_shift_px": 0.0, "pslr_diff_db": 0.0, "islr_diff_db": 0.0, "targets": []}
    for (x, y) in pixels:
        a = point_target(img, int(x), int(y))
        b = point_target(ref, int(x), int(y))
        shift = float(np.hypot(a.x - b.x, a.y - b.y))
        dp = max(abs(a.pslr_range_db - b.pslr_range_db), abs(a.pslr_azimuth_db - b.pslr_azimuth_db))
        di = max(abs(a.islr_range_db - b.islr_range_db), abs(a.islr_azimuth_db - b.islr_azimuth_db))
        out["peak_shift_px"] = max(out["peak_shift_px"], shift)
        out["pslr_diff_db"] = max(out["pslr_diff_db"], dp)
        out["islr_diff_db"] = max(out["islr_diff_db"], di)
        out["targets"].append({"x": x, "y": y, "img": dataclasses.asdict(a), "ref": dataclasses.asdict(b)})
    return out


def target_pixels(scene) -> list:
    """Nearest pixel (x, y) of each target of a scene whose grid is axis-aligned."""
    g = scene.grid
    M = np.column_stack([g.ux, g.uy])  # 3x2
    out = []
    for t in scene.targets:
        d = t[:3] - g.origin
        xy, *_ = np.linalg.lstsq(M, d, rcond=None)
        x, y = int(round(xy[0])), int(round(xy[1]))
        if 0 <= x < g.nx and 0 <= y < g.ny:
            out.append((x, y))
    return out
