"""ctypes binding of libsarbp.so (include/sarbp.h) and a small Pythonic layer.

The library is the product: every call here goes through the C ABI into the
CUDA kernels.  There is no CPU fallback; importing works without a GPU, but
creating a :class:`Context` fails loudly unless an sm_103 device and the built
library are present.

Arrays may be numpy arrays (host memory: the call is synchronous) or any
object exposing ``data_ptr()`` (e.g. torch CUDA tensors: the call is
asynchronous on the given stream).
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import scenes

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libsarbp.so")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_UNSUPPORTED = 2
ERR_OUT_OF_MEMORY = 3
ERR_CUDA = 4
ERR_NO_DEVICE = 5
ERR_TIMEOUT = 6
ERR_DEVICE_CHECK = 7
ERR_NOT_READY = 8
ERR_CANCELLED = 9
ERR_BUDGET = 10
ERR_INTERNAL = 11

MODE_FP64 = 0
MODE_FP32 = 1
MODE_SPLIT = 2
MODE_FP16STORE = 3
MODES = {"fp64": MODE_FP64, "fp32": MODE_FP32, "split": MODE_SPLIT, "fp16store": MODE_FP16STORE}

STORE_C64 = 0
STORE_C32H = 1


class Radar(ctypes.Structure):
    _fields_ = [("c", ctypes.c_double), ("fc", ctypes.c_double), ("fs", ctypes.c_double),
                ("kr", ctypes.c_double), ("tp", ctypes.c_double), ("tc", ctypes.c_double),
                ("t_rec0", ctypes.c_double), ("upsample", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Grid(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("ux", ctypes.c_double * 3), ("uy", ctypes.c_double * 3),
                ("nx", ctypes.c_int32), ("ny", ctypes.c_int32)]


class RcLayout(ctypes.Structure):
    _fields_ = [("nc", ctypes.c_int32), ("nfft", ctypes.c_int32), ("shift", ctypes.c_int32),
                ("nbins", ctypes.c_int32), ("t0_bins", ctypes.c_double), ("bin_rate", ctypes.c_double)]


class WkParams(ctypes.Structure):
    _fields_ = [("fr", ctypes.c_double), ("prf", ctypes.c_double), ("f0", ctypes.c_double),
                ("r0", ctypes.c_double), ("kr", ctypes.c_double), ("c", ctypes.c_double),
                ("vr", ctypes.c_double), ("f_nc", ctypes.c_double), ("taps", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


def wk_params(p) -> WkParams:
    """WkParams from any object with fr, prf, f0, r0, kr, c, vr, f_nc, taps."""
    w = WkParams()
    for f in ("fr", "prf", "f0", "r0", "kr", "c", "vr", "f_nc"):
        setattr(w, f, float(getattr(p, f)))
    w.taps = int(p.taps)
    return w


class CeosLayout(ctypes.Structure):
    _fields_ = [("file_header", ctypes.c_int32), ("header", ctypes.c_int32), ("aux", ctypes.c_int32),
                ("cells", ctypes.c_int32), ("replica", ctypes.c_int32), ("replica_line", ctypes.c_int32),
                ("lines_per_block", ctypes.c_int32), ("agc_byte", ctypes.c_int32), ("gain", ctypes.c_float),
                ("reserved", ctypes.c_int32)]


def ceos_layout(l=None) -> CeosLayout:
    """CeosLayout from an object with the same field names (RADARSAT-1 values by default)."""
    c = CeosLayout(16252, 192, 50, 9288, 2880, 7, 8, 50, 1.5, 0)
    if l is not None:
        for f, _ in CeosLayout._fields_[:-1]:
            setattr(c, f, getattr(l, f))
    return c


class PulseCorr(ctypes.Structure):
    _fields_ = [("drange", ctypes.c_void_p), ("dphase", ctypes.c_void_p)]


class RcView(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("scale", ctypes.c_void_p), ("storage", ctypes.c_int32),
                ("np", ctypes.c_int32), ("nbins", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("t0_bins", ctypes.c_double), ("bin_rate", ctypes.c_double)]


class BpPlanInfo(ctypes.Structure):
    _fields_ = [("tile_x", ctypes.c_int32), ("tile_y", ctypes.c_int32), ("window", ctypes.c_int32),
                ("series_terms", ctypes.c_int32), ("segments", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("pulse_chunk", ctypes.c_int32), ("linear_phase", ctypes.c_int32), ("smem_bytes", ctypes.c_uint64), ("rmin", ctypes.c_double), ("rmax", ctypes.c_double),
                ("cos_x", ctypes.c_double), ("cos_y", ctypes.c_double)]


class Target(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double), ("amp", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_jobs", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_uint64),
                ("pulses_per_step", ctypes.c_int32), ("use_graphs", ctypes.c_int32),
                ("step_updates", ctypes.c_uint64)]


class Job(ctypes.Structure):
    _fields_ = [("radar", Radar), ("grid", Grid), ("echo", ctypes.c_void_p), ("apc", ctypes.c_void_p),
                ("image", ctypes.c_void_p), ("np", ctypes.c_int32), ("ns", ctypes.c_int32),
                ("mode", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class JobStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("steps", ctypes.c_int32), ("queued_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double), ("updates", ctypes.c_double), ("device_bytes", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "rejected", "cancelled",
                                               "steps", "graph_launches")] + \
               [("updates", ctypes.c_double), ("busy_s", ctypes.c_double), ("bytes_in_use", ctypes.c_uint64),
                ("peak_bytes", ctypes.c_uint64), ("active", ctypes.c_int32), ("queued", ctypes.c_int32),
                ("peak_active", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("step_device_s", ctypes.c_double), ("admit_device_s", ctypes.c_double)]


class RefParams(ctypes.Structure):
    """Byte layout of the reference's SARParams (code/SAR_BP/CUDA/BPA_CUDA.h:28-50)."""
    _fields_ = [(n, ctypes.c_float) for n in ("c", "fc", "lam", "Kr", "Tr", "Br", "Fr", "vr", "H", "La",
                                              "Rg0", "Az0")] + \
               [("Nfast", ctypes.c_int32), ("Mslow", ctypes.c_int32), ("Ntarget", ctypes.c_int32)]

    @classmethod
    def defaults(cls) -> "RefParams":
        """The reference's default-constructed SARParams (BPA_CUDA.h:29-49)."""
        p = cls()
        p.c, p.fc = 3e8, 5.3e9
        p.lam = np.float32(p.c) / np.float32(p.fc)
        p.Kr, p.Tr, p.Br, p.Fr = 4e12, 2.5e-6, 1e8, 1.2e8
        p.vr, p.H, p.La, p.Rg0, p.Az0 = 150.0, 5000.0, 4.0, 10000.0, 0.0
        p.Nfast = int(np.float32(p.Tr) * np.float32(p.Fr))
        p.Mslow = 1024
        p.Ntarget = 5
        return p


SIGNATURES = {
    "sarbp_abi_version": ([], ctypes.c_int),
    "sarbp_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "sarbp_create": ([ctypes.POINTER(ctypes.c_void_p), ctypes.c_int], ctypes.c_int),
    "sarbp_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "sarbp_last_error": ([ctypes.c_void_p], ctypes.c_char_p),
    "sarbp_synchronize": ([ctypes.c_void_p], ctypes.c_int),
    "sarbp_trim": ([ctypes.c_void_p], ctypes.c_int),
    "sarbp_device_bytes": ([ctypes.c_void_p], ctypes.c_size_t),
    "sarbp_rc_layout_get": ([ctypes.POINTER(Radar), ctypes.c_int32, ctypes.POINTER(RcLayout)], ctypes.c_int),
    "sarbp_range_compress": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.c_void_p, ctypes.c_int32,
                              ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p], ctypes.c_int),
    "sarbp_range_compress_noalloc": ([ctypes.POINTER(Radar), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                                     ctypes.c_int),
    "sarbp_backproject": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.POINTER(RcView), ctypes.c_void_p,
                           ctypes.POINTER(Grid), ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                           ctypes.c_void_p], ctypes.c_int),
    "sarbp_backproject_ex": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.POINTER(RcView), ctypes.c_void_p,
                              ctypes.POINTER(Grid), ctypes.c_int32, ctypes.POINTER(PulseCorr), ctypes.c_void_p,
                              ctypes.c_int32, ctypes.c_void_p], ctypes.c_int),
    "sarbp_bp_plan": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.POINTER(RcView), ctypes.c_void_p,
                       ctypes.POINTER(Grid), ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(BpPlanInfo)], ctypes.c_int),
    "sarbp_project_weighted": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.POINTER(RcView), ctypes.c_void_p,
                                ctypes.POINTER(Grid), ctypes.c_int32, ctypes.POINTER(PulseCorr), ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "sarbp_autofocus": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.POINTER(RcView), ctypes.c_void_p,
                         ctypes.POINTER(Grid), ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "sarbp_wk_padded_size": ([ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                              ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
    "sarbp_wk_image": ([ctypes.c_void_p, ctypes.POINTER(WkParams), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                        ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "sarbp_wk_preprocess": ([ctypes.c_void_p, ctypes.POINTER(WkParams), ctypes.c_void_p, ctypes.c_int32,
                             ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "sarbp_wk_focus": ([ctypes.c_void_p, ctypes.POINTER(WkParams), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                        ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "sarbp_dft": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p],
                  ctypes.c_int),
    "sarbp_dft2d": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p],
                  ctypes.c_int),
    "sarbp_ceos_decode": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(CeosLayout),
                           ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "sarbp_image": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                     ctypes.c_void_p, ctypes.POINTER(Grid), ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p],
                    ctypes.c_int),
    "sarbp_synthesize_echo": ([ctypes.c_void_p, ctypes.POINTER(Radar), ctypes.c_void_p, ctypes.c_int32,
                               ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_uint64,
                               ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "sarbp_server_create": ([ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ServerConfig)], ctypes.c_int),
    "sarbp_server_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "sarbp_server_submit": ([ctypes.c_void_p, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "sarbp_server_poll": ([ctypes.c_void_p, ctypes.c_uint64], ctypes.c_int),
    "sarbp_server_wait": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(JobStats)],
                          ctypes.c_int),
    "sarbp_server_cancel": ([ctypes.c_void_p, ctypes.c_uint64], ctypes.c_int),
    "sarbp_server_get_stats": ([ctypes.c_void_p, ctypes.POINTER(ServerStats)], ctypes.c_int),
    "sarbp_server_debug_set": ([ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64], ctypes.c_int),
    "sarbp_launch_back_projection": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(RefParams),
                                      ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "sarbp_launch_generate_echo": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.POINTER(RefParams), ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "sarbp_probe_issue_rates": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
    "sarbp_last_timings": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
                           ctypes.c_int),
    "sarbp_kernel_launches": ([ctypes.c_void_p], ctypes.c_int64),
    "sarbp_debug_set": ([ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64], ctypes.c_int),
    "sarbp_debug_get": ([ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
}

# sarbp_debug_set / sarbp_debug_get keys (tests and tuning sweeps)
DEBUG_BP_CHUNK = 1
DEBUG_BP_SEGMENTS = 2
DEBUG_BP_CHECKED = 3
DEBUG_WAIT_LIMIT_NS = 4
DEBUG_WAIT_FAULT_CHUNK = 5
DEBUG_DEVICE_FLAGS = 6
DEBUG_BP_LINEAR_PHASE = 7
SERVER_DEBUG_FAIL_ADMIT_TICKET = 1

ABI_VERSION = 2  # SARBP_ABI_VERSION of the include/sarbp.h these bindings follow

_lib = None


def load(path: str = LIB_PATH):
    """Load libsarbp.so; raises if it has not been built or was built from
    another ABI version than these bindings."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(path)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        if L.sarbp_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{path} has ABI version {L.sarbp_abi_version()}, these bindings {ABI_VERSION}: "
                               "rebuild the library")
        _lib = L
    return _lib


class SarbpError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def _ptr(a):
    """Raw address of a numpy array or of a tensor exposing data_ptr()."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return int(a.data_ptr())
    if isinstance(a, int):
        return a
    raise TypeError(f"unsupported buffer type {type(a)}")


def radar_struct(radar: scenes.Radar, t_rec0: float, tc: float | None = None) -> Radar:
    r = Radar()
    r.c, r.fc, r.fs, r.kr, r.tp = radar.c, radar.fc, radar.fs, radar.kr, radar.tp
    r.tc = radar.tp / 2.0 if tc is None else tc
    r.t_rec0 = t_rec0
    r.upsample = radar.upsample
    r.reserved = 0
    return r


def grid_struct(g: scenes.Grid) -> Grid:
    s = Grid()
    for i in range(3):
        s.origin[i], s.ux[i], s.uy[i] = float(g.origin[i]), float(g.ux[i]), float(g.uy[i])
    s.nx, s.ny = int(g.nx), int(g.ny)
    return s


def targets_struct(tg: np.ndarray):
    arr = (Target * max(1, len(tg)))()
    for i, t in enumerate(tg):
        arr[i].x, arr[i].y, arr[i].z, arr[i].amp = (float(v) for v in t[:4])
    return arr


class Context:
    """One libsarbp context on one device (not thread-safe)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        st = self.lib.sarbp_create(ctypes.byref(h), device)
        if st != OK:
            raise SarbpError(st, f"sarbp_create(device={device}) failed: "
                                 f"{self.lib.sarbp_status_string(st).decode()}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.sarbp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, st: int, what: str):
        if st != OK:
            detail = self.lib.sarbp_last_error(self.h).decode()
            raise SarbpError(st, f"{what}: {self.lib.sarbp_status_string(st).decode()}: {detail}")

    # ---------------------------------------------------------------- calls
    def layout(self, radar: Radar, ns: int) -> RcLayout:
        lay = RcLayout()
        self.check(self.lib.sarbp_rc_layout_get(ctypes.byref(radar), ns, ctypes.byref(lay)), "rc_layout")
        return lay

    def range_compress(self, radar: Radar, echo, storage: int = STORE_C64, out=None, scale=None, stream=None):
        np_, ns = echo.shape
        lay = self.layout(radar, ns)
        if out is None:
            out = np.zeros((np_, lay.nbins), dtype=np.complex64 if storage == STORE_C64 else np.float16)
            if storage == STORE_C32H:
                out = np.zeros((np_, lay.nbins, 2), dtype=np.float16)
        if storage == STORE_C32H and scale is None:
            scale = np.zeros(np_, dtype=np.float32)
        self.check(self.lib.sarbp_range_compress(self.h, ctypes.byref(radar), _ptr(echo), np_, ns, storage,
                                                 _ptr(out), _ptr(scale), stream), "range_compress")
        return (out, scale) if storage == STORE_C32H else out

    @staticmethod
    def _rc_view(rc, scale, t0_bins: float, bin_rate: float) -> RcView:
        v = RcView()
        if isinstance(rc, np.ndarray) and rc.dtype == np.float16:
            v.storage = STORE_C32H
            v.np, v.nbins = rc.shape[0], rc.shape[1]
        else:
            v.storage = STORE_C64 if scale is None else STORE_C32H
            v.np, v.nbins = int(rc.shape[0]), int(rc.shape[1])
        v.data = _ptr(rc)
        v.scale = _ptr(scale)
        v.t0_bins, v.bin_rate = t0_bins, bin_rate
        return v

    @staticmethod
    def _corr(drange, dphase):
        if drange is None and dphase is None:
            return None, ()
        keep = tuple(None if a is None else (a if not isinstance(a, np.ndarray)
                                             else np.ascontiguousarray(a, dtype=np.float64))
                     for a in (drange, dphase))
        c = PulseCorr()
        c.drange, c.dphase = _ptr(keep[0]), _ptr(keep[1])
        return c, keep

    def backproject(self, radar: Radar, rc, apc, grid: Grid, mode: int, t0_bins: float, bin_rate: float,
                    scale=None, image=None, accumulate: bool = False, stream=None, drange=None, dphase=None):
        v = self._rc_view(rc, scale, t0_bins, bin_rate)
        if image is None:
            image = np.zeros((grid.ny, grid.nx), dtype=np.complex64)
        corr, _keep = self._corr(drange, dphase)
        if corr is None:
            self.check(self.lib.sarbp_backproject(self.h, ctypes.byref(radar), ctypes.byref(v), _ptr(apc),
                                                  ctypes.byref(grid), mode, _ptr(image), int(accumulate), stream),
                       "backproject")
        else:
            self.check(self.lib.sarbp_backproject_ex(self.h, ctypes.byref(radar), ctypes.byref(v), _ptr(apc),
                                                     ctypes.byref(grid), mode, ctypes.byref(corr), _ptr(image),
                                                     int(accumulate), stream), "backproject_ex")
        return image

    def bp_plan(self, radar: Radar, rc_view: RcView, apc, grid: Grid, mode: int, host_reduction: bool = False):
        """The tile, staging window, series terms, segments, shared memory and
        resident CTAs per SM sarbp_backproject would use (BpPlanInfo)."""
        info = BpPlanInfo()
        self.check(self.lib.sarbp_bp_plan(self.h, ctypes.byref(radar), ctypes.byref(rc_view), _ptr(apc),
                                          ctypes.byref(grid), mode, int(host_reduction), ctypes.byref(info)),
                   "bp_plan")
        return info

    def project_weighted(self, radar: Radar, rc, apc, grid: Grid, mode: int, t0_bins: float, bin_rate: float,
                         weight, scale=None, drange=None, dphase=None, out=None, stream=None):
        """out[p] = sum over pixels of conj(weight) * pulse p's term (complex128 [np])."""
        v = self._rc_view(rc, scale, t0_bins, bin_rate)
        if out is None:
            out = np.zeros(v.np, dtype=np.complex128)
        corr, _keep = self._corr(drange, dphase)
        self.check(self.lib.sarbp_project_weighted(self.h, ctypes.byref(radar), ctypes.byref(v), _ptr(apc),
                                                   ctypes.byref(grid), mode,
                                                   ctypes.byref(corr) if corr is not None else None,
                                                   _ptr(weight), _ptr(out), stream), "project_weighted")
        return out

    def autofocus(self, radar: Radar, rc, apc, grid: Grid, mode: int, t0_bins: float, bin_rate: float,
                  iterations: int, scale=None, dphase=None, drange=None, image=None, stream=None):
        """Sharpness autofocus: returns (dphase [np], sharpness [iterations + 1], image)."""
        v = self._rc_view(rc, scale, t0_bins, bin_rate)
        ph = np.zeros(v.np) if dphase is None else np.array(dphase, dtype=np.float64)
        dr = None if drange is None else np.ascontiguousarray(drange, dtype=np.float64)
        sharp = np.zeros(iterations + 1)
        if image is None:
            image = np.zeros((grid.ny, grid.nx), dtype=np.complex64)
        self.check(self.lib.sarbp_autofocus(self.h, ctypes.byref(radar), ctypes.byref(v), _ptr(apc),
                                            ctypes.byref(grid), mode, int(iterations), _ptr(dr), _ptr(ph),
                                            _ptr(image), _ptr(sharp), stream), "autofocus")
        return ph, sharp, image

    def wk_padded_size(self, na: int, nr: int):
        a, b = ctypes.c_int32(), ctypes.c_int32()
        st = self.lib.sarbp_wk_padded_size(int(na), int(nr), ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value, st

    def wk_image(self, params, echo, image=None, stream=None):
        """Omega-K image [na_pad][nr_pad] complex64 of echo [na][nr]."""
        w = params if isinstance(params, WkParams) else wk_params(params)
        na, nr = echo.shape
        NA, NR, _ = self.wk_padded_size(na, nr)
        if image is None:
            image = np.zeros((NA, NR), dtype=np.complex64)
        self.check(self.lib.sarbp_wk_image(self.h, ctypes.byref(w), _ptr(echo), na, nr, _ptr(image), stream),
                   "wk_image")
        return image

    def wk_preprocess(self, params, echo, stream=None):
        """Zero-padded, azimuth down-converted echo [na_pad][nr_pad] complex64."""
        w = params if isinstance(params, WkParams) else wk_params(params)
        na, nr = echo.shape
        NA, NR, _ = self.wk_padded_size(na, nr)
        out = np.zeros((NA, NR), dtype=np.complex64)
        self.check(self.lib.sarbp_wk_preprocess(self.h, ctypes.byref(w), _ptr(echo), na, nr, _ptr(out), stream),
                   "wk_preprocess")
        return out

    def wk_focus(self, params, spectrum, stream=None):
        """Reference-function multiply + Stolt mapping of a 2-D spectrum [na_pad][nr_pad]."""
        w = params if isinstance(params, WkParams) else wk_params(params)
        NA, NR = spectrum.shape
        out = np.zeros((NA, NR), dtype=np.complex64)
        self.check(self.lib.sarbp_wk_focus(self.h, ctypes.byref(w), _ptr(spectrum), NA, NR, _ptr(out), stream),
                   "wk_focus")
        return out

    def ceos_decode(self, raw, first_line: int, nlines: int, first_cell: int, ncells: int, layout=None,
                    apply_agc: bool = True, stream=None):
        """(echo [nlines][ncells] complex64, AGC dB [nlines] int16) from CEOS file bytes."""
        lay = ceos_layout(layout)
        echo = np.zeros((nlines, ncells), dtype=np.complex64)
        agc = np.zeros(nlines, dtype=np.int16)
        nbytes = raw.nbytes if isinstance(raw, np.ndarray) else raw.numel() * raw.element_size()
        self.check(self.lib.sarbp_ceos_decode(self.h, _ptr(raw), nbytes, ctypes.byref(lay), first_line, nlines,
                                              first_cell, ncells, int(apply_agc), _ptr(echo), _ptr(agc), stream),
                   "ceos_decode")
        return echo, agc

    def dft(self, data, inverse: bool = False, stream=None):
        """In-place batched DFT along the rows of data [rows][n] (complex64)."""
        rows, n = data.shape
        self.check(self.lib.sarbp_dft(self.h, _ptr(data), rows, n, int(inverse), stream), "dft")
        return data

    def dft2d(self, data, inverse: bool = False, stream=None):
        """In-place 2-D DFT of data [na][nr] (complex64): rows, then columns."""
        na, nr = data.shape
        self.check(self.lib.sarbp_dft2d(self.h, _ptr(data), na, nr, int(inverse), stream), "dft2d")
        return data

    def image(self, radar: Radar, echo, apc, grid: Grid, mode: int, image=None, stream=None):
        np_, ns = echo.shape
        if image is None:
            image = np.zeros((grid.ny, grid.nx), dtype=np.complex64)
        self.check(self.lib.sarbp_image(self.h, ctypes.byref(radar), _ptr(echo), np_, ns, _ptr(apc),
                                        ctypes.byref(grid), mode, _ptr(image), stream), "image")
        return image

    def synthesize_echo(self, radar: Radar, apc, ns: int, targets: np.ndarray, snr_db=None, seed: int = 0,
                        out=None, stream=None):
        apc_a = apc
        np_ = int(apc.shape[0])
        tg = targets_struct(targets)
        if out is None:
            out = np.zeros((np_, ns), dtype=np.complex64)
        snr = float("nan") if snr_db is None else float(snr_db)
        self.check(self.lib.sarbp_synthesize_echo(self.h, ctypes.byref(radar), _ptr(apc_a), np_, ns,
                                                  ctypes.cast(tg, ctypes.c_void_p), len(targets), snr,
                                                  ctypes.c_uint64(seed & (2**64 - 1)), _ptr(out), stream),
                   "synthesize_echo")
        return out

    def synchronize(self):
        self.check(self.lib.sarbp_synchronize(self.h), "synchronize")

    def trim(self):
        """Release the context's cached device buffers."""
        self.check(self.lib.sarbp_trim(self.h), "trim")

    def timings(self):
        a, b = ctypes.c_float(), ctypes.c_float()
        self.check(self.lib.sarbp_last_timings(self.h, ctypes.byref(a), ctypes.byref(b)), "timings")
        return a.value, b.value

    def launches(self) -> int:
        return int(self.lib.sarbp_kernel_launches(self.h))

    def debug_set(self, key: int, value: int):
        """Test / tuning switch of this context (sarbp_debug_set)."""
        self.check(self.lib.sarbp_debug_set(self.h, int(key), int(value)), "debug_set")

    def debug_get(self, key: int) -> int:
        v = ctypes.c_int64()
        self.check(self.lib.sarbp_debug_get(self.h, int(key), ctypes.byref(v)), "debug_get")
        return int(v.value)

    def probe_issue_rates(self):
        f, m, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        self.check(self.lib.sarbp_probe_issue_rates(self.h, ctypes.byref(f), ctypes.byref(m), ctypes.byref(n)),
                   "probe")
        return f.value, m.value, n.value


# --------------------------------------------------------- scene helpers --

def scene_args(scene: scenes.Scene):
    """(radar struct, grid struct, layout) for a synthetic scene."""
    r = radar_struct(scene.radar, scene.t_rec0)
    return r, grid_struct(scene.grid), scene.layout


def synthesize(ctx: Context, scene: scenes.Scene, out=None, stream=None):
    r = radar_struct(scene.radar, scene.t_rec0)
    return ctx.synthesize_echo(r, scene.apc, scene.ns, scene.targets, scene.snr_db, scene.seed, out=out,
                               stream=stream)


def image_scene(ctx: Context, scene: scenes.Scene, echo, mode: int, image=None, stream=None):
    r, g, _ = scene_args(scene)
    return ctx.image(r, echo, scene.apc, g, mode, image=image, stream=stream)


def nan_to_none(x):
    return None if x is None or (isinstance(x, float) and math.isnan(x)) else x


class Server:
    """Continuous-batching imaging service (sarbp_server_* in include/sarbp.h)."""

    def __init__(self, device: int = 0, max_jobs: int = 16, hbm_budget_bytes: int = 64 << 30,
                 pulses_per_step: int = 512, use_graphs: bool = True, step_updates: int = 0):
        self.lib = load()
        cfg = ServerConfig(device, max_jobs, hbm_budget_bytes, pulses_per_step, int(use_graphs), int(step_updates))
        h = ctypes.c_void_p()
        st = self.lib.sarbp_server_create(ctypes.byref(h), ctypes.byref(cfg))
        if st != OK:
            raise SarbpError(st, f"sarbp_server_create: {self.lib.sarbp_status_string(st).decode()}")
        self.h = h
        self._keep = {}  # ticket -> buffers that must outlive the job

    def close(self):
        if getattr(self, "h", None):
            self.lib.sarbp_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, radar: Radar, grid: Grid, echo, apc, mode: int = MODE_SPLIT, image=None) -> int:
        """echo: numpy complex64 [np][ns], or a (pinned) float32 tensor [np][2 ns]."""
        if isinstance(echo, np.ndarray):
            if echo.dtype != np.complex64 or echo.ndim != 2:
                raise ValueError("echo must be complex64 [np][ns]")
            np_, ns = echo.shape
        else:
            np_, ns = int(echo.shape[0]), int(echo.shape[1]) // 2
        if image is None:
            image = np.zeros((grid.ny, grid.nx), dtype=np.complex64)
        apc = np.ascontiguousarray(apc, dtype=np.float64)
        j = Job()
        j.radar, j.grid = radar, grid
        j.echo, j.apc, j.image = _ptr(echo), _ptr(apc), _ptr(image)
        j.np, j.ns, j.mode = np_, ns, mode
        t = ctypes.c_uint64()
        st = self.lib.sarbp_server_submit(self.h, ctypes.byref(j), ctypes.byref(t))
        if st != OK:
            raise SarbpError(st, f"submit: {self.lib.sarbp_status_string(st).decode()}")
        self._keep[t.value] = (echo, apc, image)
        return t.value

    def poll(self, ticket: int) -> int:
        return self.lib.sarbp_server_poll(self.h, ticket)

    def cancel(self, ticket: int) -> int:
        return self.lib.sarbp_server_cancel(self.h, ticket)

    def wait(self, ticket: int, timeout_ms: int = -1):
        """Returns (status, JobStats, image)."""
        s = JobStats()
        st = self.lib.sarbp_server_wait(self.h, ticket, timeout_ms, ctypes.byref(s))
        if st == ERR_TIMEOUT:
            return st, s, None
        _, _, image = self._keep.pop(ticket, (None, None, None))
        return st, s, image

    def debug_set(self, key: int, value: int):
        """Test switch of this server (sarbp_server_debug_set)."""
        st = self.lib.sarbp_server_debug_set(self.h, int(key), int(value))
        if st != OK:
            raise SarbpError(st, "server debug_set")

    def stats(self) -> ServerStats:
        s = ServerStats()
        st = self.lib.sarbp_server_get_stats(self.h, ctypes.byref(s))
        if st != OK:
            raise SarbpError(st, "stats")
        return s
