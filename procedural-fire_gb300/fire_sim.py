"""Python host mirror of the reference's FireSim (src/sim.js) over the C ABI in include/fire_sim.h.

The reference drives its simulation from JavaScript: ``new FireSim(device, {res, size, logs, vcycles})``,
``sim.step(enc, dt)``, ``sim.setParams({...})``, ``sim.reset()``, and the page API's events and
diagnostics (src/main.js ``window.FIRE``).  This module exposes the same surface with the same names,
argument meanings and error behaviour, backed by the CUDA sm_103a library ``libfiresim.so``.

There is no CPU fallback: constructing a FireSim without the built library or without a GB300-class
device raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path
from typing import Dict, Iterable, Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libfiresim.so"

# SIM_FIELDS (src/sim.js:14-23)
SIM_FIELDS = [
    "nx", "ny", "nz", "dx", "dt", "time", "frame", "seed",
    "ox", "oy", "oz", "nLogs",
    "fuelSrc", "bedFuel", "srcTemp", "bedTemp", "srcVel", "srcFreq", "srcSpeed", "srcThresh",
    "ignT", "kMix", "rs", "heatOut", "expansion", "sootForm", "sootOx", "radCool",
    "coolRate", "sootDissip", "smokeDissip", "vitDecay", "fuelDissip", "buoyancy", "vortEps", "turbAmp",
    "turbFreq", "turbRise", "turbEvolve", "windX", "windZ", "gust", "intensity", "velDissip",
    "bedRadius", "logSrc", "burstX", "burstY", "burstZ", "burstAmt", "smolder", "sponge", "hotR0", "hotR1", "hotY1",
    "visc", "lamAge", "anchorFreq", "srcFloor", "anchorGain",
]
# Fields (src/sim.js:71-76 texture names; p/b = multigrid level 0)
FIELDS = {"vel": 0, "velX": 1, "velY": 2, "S": 3, "SX": 4, "SY": 5, "S2": 6, "S2X": 7, "S2Y": 8,
          "vort": 9, "geo": 10, "p": 11, "b": 12, "noise": 13, "curl": 14}
STAGES = {"geo": 0, "adv1": 1, "adv2": 2, "curl": 3, "forces": 4, "div": 5, "vcycle": 6, "project": 7}
ERRORS = {1: "bad argument", 2: "unknown parameter", 3: "CUDA error", 4: "no sm_103 device", 5: "out of memory",
          6: "bad state"}


class FireError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class FireConfig(ctypes.Structure):
    _fields_ = [("res", ctypes.c_int * 3), ("size", ctypes.c_float * 3), ("vcycles", ctypes.c_int),
                ("device", ctypes.c_int), ("noise_seed", ctypes.c_int), ("mg_max_cycles", ctypes.c_int),
                ("mg_tol", ctypes.c_double)]


class FireFieldDesc(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dims", ctypes.c_int * 3), ("channels", ctypes.c_int),
                ("elem_bytes", ctypes.c_int), ("strides", ctypes.c_size_t * 3), ("bytes", ctypes.c_size_t)]


class FireInfo(ctypes.Structure):
    _fields_ = [("res", ctypes.c_int * 3), ("size", ctypes.c_float * 3), ("dx", ctypes.c_float),
                ("origin", ctypes.c_float * 3), ("time", ctypes.c_double), ("frame", ctypes.c_longlong),
                ("n_levels", ctypes.c_int), ("coarse_iters", ctypes.c_int), ("vcycles", ctypes.c_int),
                ("last_cycles", ctypes.c_int), ("last_rel_residual", ctypes.c_double),
                ("total_cycles", ctypes.c_longlong)]


# Every exported entry point and its ctypes signature (mirrors include/fire_sim.h).
_vp, _ip, _fp, _dp, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_size_t
_SIGS = {
    "fire_sim_create": (_ip, [ctypes.POINTER(FireConfig), _vp, _ip, ctypes.POINTER(_vp)]),
    "fire_sim_destroy": (_ip, [_vp]),
    "fire_sim_step": (_ip, [_vp, _fp, _ip, _vp]),
    "fire_sim_sync": (_ip, [_vp]),
    "fire_sim_set_params": (_ip, [_vp, ctypes.POINTER(ctypes.c_char_p), _vp, _ip]),
    "fire_sim_get_param": (_ip, [_vp, ctypes.c_char_p, ctypes.POINTER(_fp)]),
    "fire_sim_set_param_block": (_ip, [_vp, _vp]),
    "fire_sim_get_param_block": (_ip, [_vp, _vp]),
    "fire_sim_peek_block": (_ip, [_vp, _fp, _vp]),
    "fire_param_index": (_ip, [ctypes.c_char_p]),
    "fire_param_name": (ctypes.c_char_p, [_ip]),
    "fire_param_defaults": (_ip, [_vp]),
    "fire_sim_set_soot_age": (_ip, [_vp, _fp, _fp]),
    "fire_sim_set_bed_gain": (_ip, [_vp, _fp]),
    "fire_sim_set_spots": (_ip, [_vp, _vp, _ip]),
    "fire_sim_inject": (_ip, [_vp, _fp, _fp, _fp, _fp, _fp]),
    "fire_sim_stoke": (_ip, [_vp, _ip, _fp]),
    "fire_sim_gust": (_ip, [_vp, _fp, _fp]),
    "fire_sim_reset": (_ip, [_vp]),
    "fire_sim_upload_logs": (_ip, [_vp, _vp, _ip]),
    "fire_sim_field": (_ip, [_vp, _ip, ctypes.POINTER(FireFieldDesc)]),
    "fire_sim_download": (_ip, [_vp, _ip, _vp, _sz]),
    "fire_sim_upload": (_ip, [_vp, _ip, _vp, _sz]),
    "fire_sim_info": (_ip, [_vp, ctypes.POINTER(FireInfo)]),
    "fire_sim_last_error": (ctypes.c_char_p, [_vp]),
    "fire_sim_run_stage": (_ip, [_vp, _ip, _fp, _vp]),
    "fire_sim_run_mg": (_ip, [_vp, _ip, _ip, _ip, _vp]),
    "fire_sim_level_io": (_ip, [_vp, _ip, _ip, _vp, _sz, _ip]),
    "fire_sim_level_dims": (_ip, [_vp, _ip, ctypes.POINTER(_ip), ctypes.POINTER(_fp)]),
    "fire_sim_profile": (_ip, [_vp, _ip]),
    "fire_sim_stage_times": (_ip, [_vp, _vp, _ip]),
    "fire_sim_residual": (_ip, [_vp, ctypes.POINTER(_dp), _vp]),
    "fire_sim_stats": (_ip, [_vp, _ip, _vp, _vp]),
    "fire_sim_hrr": (_ip, [_vp, ctypes.POINTER(_dp), _vp]),
    "fire_sim_stats_async": (_ip, [_vp, _vp, _vp]),
    "fire_sim_set_step_stats": (_ip, [_vp, _ip]),
    "fire_sim_height_profile": (_ip, [_vp, _vp, _ip, ctypes.POINTER(_ip), _vp]),
    "fire_build_campfire": (_ip, [ctypes.c_uint32, _vp, _ip]),
    "fire_make_spots": (_ip, [ctypes.c_uint32, _ip, _fp, _fp, _fp, _fp, _vp]),
    "fire_poisson_vcycles_noalloc": (_ip, [_vp, _vp, _ip, _ip, _ip, _fp, _ip, _vp]),
    "fire_poisson_noalloc_status": (_ip, [_vp]),
    "fire_sparks_create": (_ip, [_vp, _ip, ctypes.POINTER(_vp)]),
    "fire_sparks_destroy": (_ip, [_vp]),
    "fire_sparks_reset": (_ip, [_vp]),
    "fire_sparks_burst": (_ip, [_vp, _ip, _vp, _fp, _fp, _fp, _fp, _fp, _vp]),
    "fire_sparks_set": (_ip, [_vp, _fp, _fp, _fp, _fp, _fp]),
    "fire_sparks_step": (_ip, [_vp, _fp, _vp]),
    "fire_sparks_peek": (_ip, [_vp, _fp, _vp]),
    "fire_sparks_buffer": (_ip, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_ip)]),
    "fire_sparks_io": (_ip, [_vp, _vp, _sz, _ip]),
    "fire_sparks_set_rate": (_ip, [_vp, _fp]),
    "fire_volume_create": (_ip, [_vp, _ip, _ip, _fp, _fp, ctypes.POINTER(_vp)]),
    "fire_volume_destroy": (_ip, [_vp]),
    "fire_volume_size": (_ip, [_vp, ctypes.POINTER(_ip), ctypes.POINTER(_ip)]),
    "fire_volume_set_params": (_ip, [_vp, ctypes.POINTER(ctypes.c_char_p), _vp, _ip]),
    "fire_volume_set_camera": (_ip, [_vp, _vp, _vp, _dp, _fp, _fp]),
    "fire_volume_set_depth": (_ip, [_vp, _vp, _ip, _ip]),
    "fire_volume_uniforms": (_ip, [_vp, _dp, _ip, _vp, _ip]),
    "fire_volume_render": (_ip, [_vp, _dp, _ip, _vp]),
    "fire_volume_download": (_ip, [_vp, _ip, _vp, _sz]),
    "fire_blackbody_lut": (_ip, [_ip, _fp, _fp, _fp, _vp]),
    "fire_timeline_event_count": (_ip, []),
    "fire_timeline_events": (_ip, [_vp, _ip]),
    "fire_timeline_intensity_at": (_dp, [_dp]),
    "fire_timeline_sim_at": (_ip, [_dp, _vp]),
    "fire_timeline_log_offsets_at": (_ip, [_dp, ctypes.POINTER(_ip), ctypes.POINTER(_dp), ctypes.POINTER(_dp),
                                            ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "fire_timeline_camera_at": (_ip, [_dp, _vp, _vp, ctypes.POINTER(_dp)]),
    "fire_timeline_lens_at": (_ip, [_dp, ctypes.POINTER(_dp), ctypes.POINTER(_dp), ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "fire_timeline_exposure_at": (_dp, [_dp]),
    "fire_timeline_preroll": (_dp, []),
    "fire_timeline_create": (_ip, [_vp, _ip, _ip, ctypes.POINTER(_vp)]),
    "fire_timeline_destroy": (_ip, [_vp]),
    "fire_timeline_step_dt": (_dp, [_vp]),
    "fire_timeline_step_time": (_dp, [_vp, ctypes.c_longlong]),
    "fire_timeline_step": (_ip, [_vp, _vp, _vp, ctypes.c_longlong, _vp]),
    "fire_ensemble_create": (_ip, [ctypes.POINTER(FireConfig), _ip, ctypes.POINTER(_vp)]),
    "fire_ensemble_destroy": (_ip, [_vp]),
    "fire_ensemble_size": (_ip, [_vp]),
    "fire_ensemble_sim": (_ip, [_vp, _ip, ctypes.POINTER(_vp)]),
    "fire_ensemble_step": (_ip, [_vp, _fp, _ip, _vp]),
    "fire_ensemble_sync": (_ip, [_vp]),
    "fire_ensemble_last_error": (ctypes.c_char_p, [_vp]),
    "fire_ensemble_set_autotune": (_ip, [_vp, _ip]),
    "fire_ensemble_set_tiles": (_ip, [_vp, _vp]),
    "fire_ensemble_tiles": (_ip, [_vp, _vp, _vp]),
    "fire_poisson_create": (_ip, [_vp, _fp, _ip, _ip, ctypes.POINTER(_vp)]),
    "fire_poisson_destroy": (_ip, [_vp]),
    "fire_poisson_solve": (_ip, [_vp, _vp, _vp, _vp, _dp, _ip, _ip, _vp]),
    "fire_poisson_result": (_ip, [_vp, _vp]),
    "fire_poisson_residual": (_ip, [_vp, _vp, _vp, _vp, ctypes.POINTER(_dp)]),
    "fire_poisson_make_rhs": (_ip, [_vp, _vp, ctypes.c_uint, _ip, _fp, _vp]),
    "fire_poisson_sources": (_ip, [ctypes.c_uint, _ip, _vp, _vp]),
    "fire_poisson_set_study": (_ip, [_vp, _ip]),
    "fire_adjoint_create": (_ip, [_vp, _ip, _ip, ctypes.POINTER(_vp)]),
    "fire_adjoint_destroy": (_ip, [_vp]),
    "fire_adjoint_forward": (_ip, [_vp, _fp, _vp]),
    "fire_adjoint_loss": (_ip, [_vp, _vp, ctypes.POINTER(_dp)]),
    "fire_adjoint_seed": (_ip, [_vp, _vp, _vp, _vp]),
    "fire_adjoint_backward": (_ip, [_vp, _vp]),
    "fire_adjoint_grad_spots": (_ip, [_vp, _vp, _ip]),
    "fire_adjoint_io": (_ip, [_vp, _ip, _vp, ctypes.c_size_t, _ip]),
    "fire_adjoint_clear": (_ip, [_vp]),
    "fire_adjoint_stage": (_ip, [_vp, _ip, _fp, _ip, _vp]),
    "fire_adjoint_timing": (_ip, [_vp, ctypes.POINTER(_fp), ctypes.POINTER(_fp)]),
    "fire_sim_set_mg_omega": (_ip, [_vp, _fp]),
    "fire_sim_set_tail_wait_limit": (_ip, [_vp, _ip]),
    "fire_sim_save": (_ip, [_vp, _vp, _sz, ctypes.POINTER(_sz)]),
    "fire_sim_load": (_ip, [_vp, _vp, _sz]),
    "fire_device_ok": (_ip, [_ip]),
    "fire_version": (ctypes.c_char_p, []),
}
EXPORTS = tuple(_SIGS)

_lib = None


def load_library(path: Optional[os.PathLike] = None):
    """Loads libfiresim.so; raises if it was not built (there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FireError(3, f"{p} is missing: build it with procedural-fire_gb300/fire_build.py")
    L = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def param_defaults() -> np.ndarray:
    """SIM_DEFAULTS (src/sim.js:25-44) as the 64-float block."""
    out = np.zeros(64, np.float32)
    load_library().fire_param_defaults(_ptr(out))
    return out


SIM_DEFAULTS_NAMES = SIM_FIELDS[12:]


def build_campfire(seed: int = 7, max_logs: int = 16) -> np.ndarray:
    """buildCampfire(seed) + packLogs (src/scene.js:21-98): max_logs * 8 floats."""
    out = np.zeros(max_logs * 8, np.float32)
    n = load_library().fire_build_campfire(seed, _ptr(out), max_logs)
    if n < 0:
        raise FireError(1, "build_campfire")
    return out


def make_spots(seed: int, n: int, flux_lo: float = 1.0, flux_hi: float = 4.0, sigma: float = 0.02,
               radius: float = 0.15) -> np.ndarray:
    out = np.zeros((max(n, 1), 5), np.float32)
    rc = load_library().fire_make_spots(seed, n, flux_lo, flux_hi, sigma, radius, _ptr(out))
    if rc:
        raise FireError(rc, "make_spots")
    return out[:n]


def device_ok(device: int = 0) -> bool:
    return bool(load_library().fire_device_ok(device))


def _stream_handle(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))   # torch.cuda.Stream


class FireSim:
    """GPU fire simulation with the reference FireSim's interface (src/sim.js:48-649)."""

    def __init__(self, res: Sequence[int] = (80, 120, 80), size: Sequence[float] = (1.2, 1.8, 1.2),
                 logs: Optional[np.ndarray] = None, vcycles: int = 2, device: int = 0, noise_seed: int = 1,
                 mg_max_cycles: int = 0, mg_tol: float = 0.0):
        self._lib = load_library()
        self._h = None
        cfg = FireConfig()
        cfg.res[:] = [int(r) for r in res]
        cfg.size[:] = [float(s) for s in size]
        cfg.vcycles = int(vcycles)
        cfg.device = int(device)
        cfg.noise_seed = int(noise_seed)
        cfg.mg_max_cycles = int(mg_max_cycles)
        cfg.mg_tol = float(mg_tol)
        if logs is None:
            logs = np.zeros(0, np.float32)
        lg = np.ascontiguousarray(logs, np.float32).reshape(-1)
        if lg.size % 8:
            raise FireError(1, "logs must hold 8 floats per log")
        h = ctypes.c_void_p()
        rc = self._lib.fire_sim_create(ctypes.byref(cfg), _ptr(lg) if lg.size else None, lg.size // 8, ctypes.byref(h))
        if rc:
            raise FireError(rc, "fire_sim_create")
        self._h = h
        self._owned = True
        self._describe()

    @classmethod
    def _borrow(cls, handle: ctypes.c_void_p):
        """A view of a simulation owned elsewhere (an ensemble member): never destroyed by this object."""
        self = cls.__new__(cls)
        self._lib = load_library()
        self._h = handle
        self._owned = False
        self._describe()
        return self

    def _describe(self):
        info = self.info()
        self.res = tuple(int(r) for r in info.res)
        self.size = tuple(float(s) for s in info.size)
        self.dx = info.dx
        self.origin = tuple(info.origin)
        self.coarse_iters = info.coarse_iters
        self.levels = []
        for l in range(info.n_levels):
            d = (ctypes.c_int * 3)()
            hh = ctypes.c_float()
            self._lib.fire_sim_level_dims(self._h, l, d, ctypes.byref(hh))
            self.levels.append({"dims": tuple(d), "h": hh.value})
        self._pinned = None

    # ---- lifetime ----
    def close(self):
        if self._h is not None:
            if getattr(self, "_owned", True):
                self._lib.fire_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int, what: str):
        if rc:
            msg = self._lib.fire_sim_last_error(self._h)
            raise FireError(rc, f"{what}: {msg.decode() if msg else ''}")

    # ---- stepping ----
    def step(self, dt: float, n: int = 1, stream=None):
        """FireSim.step (src/sim.js:627-648), n times, asynchronously on `stream`."""
        self._check(self._lib.fire_sim_step(self._h, float(dt), int(n), _stream_handle(stream)), "step")

    def sync(self):
        self._check(self._lib.fire_sim_sync(self._h), "sync")

    # ---- parameters ----
    def set_params(self, p: Dict[str, float]):
        """FireSim.setParams (src/sim.js:601-604); unknown names raise, as UniformStruct.set does."""
        if not p:
            return
        names = (ctypes.c_char_p * len(p))(*[k.encode() for k in p])
        vals = np.asarray(list(p.values()), np.float32)
        self._check(self._lib.fire_sim_set_params(self._h, names, _ptr(vals), len(p)), "set_params")

    setParams = set_params

    @property
    def params(self) -> Dict[str, float]:
        blk = np.zeros(64, np.float32)
        self._check(self._lib.fire_sim_get_param_block(self._h, _ptr(blk)), "params")
        return {k: float(blk[i]) for i, k in enumerate(SIM_FIELDS)}

    def peek_block(self, dt: float) -> np.ndarray:
        """The 208-float block (SIM_FIELDS uniforms + extension) the next step uploads."""
        out = np.zeros(208, np.float32)
        self._check(self._lib.fire_sim_peek_block(self._h, float(dt), _ptr(out)), "peek_block")
        return out

    def set_soot_age(self, age0: float, age1: float):
        self._check(self._lib.fire_sim_set_soot_age(self._h, age0, age1), "set_soot_age")

    def set_bed_gain(self, gain: float):
        self._check(self._lib.fire_sim_set_bed_gain(self._h, gain), "set_bed_gain")

    def save(self) -> bytes:
        """The simulation's state as a checkpoint blob (fire_sim_save)."""
        n = ctypes.c_size_t()
        self._check(self._lib.fire_sim_save(self._h, None, 0, ctypes.byref(n)), "save")
        buf = ctypes.create_string_buffer(n.value)
        self._check(self._lib.fire_sim_save(self._h, buf, n.value, ctypes.byref(n)), "save")
        return buf.raw

    def load(self, blob: bytes):
        """Restores a checkpoint made by save() on a simulation of the same grid (fire_sim_load)."""
        buf = ctypes.create_string_buffer(bytes(blob), len(blob))
        self._check(self._lib.fire_sim_load(self._h, buf, len(blob)), "load")

    def set_tail_wait_limit(self, polls: int):
        """Fault-injection hook: bound of the multigrid tail's first bulk-copy wait (0 = give up at once)."""
        self._check(self._lib.fire_sim_set_tail_wait_limit(self._h, int(polls)), "set_tail_wait_limit")

    def set_mg_omega(self, omega: float):
        """Over-relaxation of the V-cycle's fine-level smoothing (1 = the reference's Gauss-Seidel)."""
        self._check(self._lib.fire_sim_set_mg_omega(self._h, float(omega)), "set_mg_omega")

    def set_spots(self, spots: np.ndarray):
        s = np.ascontiguousarray(spots, np.float32).reshape(-1, 5)
        self._check(self._lib.fire_sim_set_spots(self._h, _ptr(s) if len(s) else None, len(s)), "set_spots")

    # ---- events ----
    def inject(self, pos: Sequence[float], amount: float = 1.0, duration: float = 0.25):
        self._check(self._lib.fire_sim_inject(self._h, *[float(v) for v in pos], float(amount), float(duration)), "inject")

    def stoke(self, log_index: int = 3, s: float = 1.0):
        self._check(self._lib.fire_sim_stoke(self._h, int(log_index), float(s)), "stoke")

    def gust(self, strength: float = 1.0, duration: float = 2.4):
        self._check(self._lib.fire_sim_gust(self._h, float(strength), float(duration)), "gust")

    # ---- state ----
    def reset(self):
        """FireSim.reset (src/sim.js:606-618)."""
        self._check(self._lib.fire_sim_reset(self._h), "reset")

    def upload_logs(self, logs: np.ndarray):
        lg = np.ascontiguousarray(logs, np.float32).reshape(-1)
        self._check(self._lib.fire_sim_upload_logs(self._h, _ptr(lg) if lg.size else None, lg.size // 8), "upload_logs")

    def info(self) -> FireInfo:
        out = FireInfo()
        self._check(self._lib.fire_sim_info(self._h, ctypes.byref(out)), "info")
        return out

    @property
    def time(self) -> float:
        return self.info().time

    @property
    def frame(self) -> int:
        return self.info().frame

    def field(self, name: str) -> FireFieldDesc:
        d = FireFieldDesc()
        self._check(self._lib.fire_sim_field(self._h, FIELDS[name], ctypes.byref(d)), f"field {name}")
        return d

    def _shape(self, d: FireFieldDesc):
        shape = (d.dims[2], d.dims[1], d.dims[0]) + ((d.channels,) if d.channels > 1 else ())
        return shape, (np.float16 if d.elem_bytes == 2 else np.float32)

    def download(self, name: str) -> np.ndarray:
        d = self.field(name)
        shape, dt = self._shape(d)
        out = np.empty(shape, dt)
        self._check(self._lib.fire_sim_download(self._h, FIELDS[name], _ptr(out), out.nbytes), f"download {name}")
        return out

    def upload(self, name: str, arr: np.ndarray):
        d = self.field(name)
        shape, dt = self._shape(d)
        a = np.ascontiguousarray(arr, dt)
        if a.size != int(np.prod(shape)):
            raise FireError(1, f"upload {name}: expected shape {shape}")
        self._check(self._lib.fire_sim_upload(self._h, FIELDS[name], _ptr(a), a.nbytes), f"upload {name}")

    # ---- stage-level ----
    def run_stage(self, name: str, dt: float, stream=None):
        self._check(self._lib.fire_sim_run_stage(self._h, STAGES[name], float(dt), _stream_handle(stream)), f"stage {name}")

    def run_mg(self, op: str, level: int, arg: int = 0, stream=None):
        code = {"smooth": 1, "restrict": 2, "prolong": 3, "tail": 4, "sweeps": 5, "residual": 6}[op]
        self._check(self._lib.fire_sim_run_mg(self._h, code, level, arg, _stream_handle(stream)), f"mg {op}")

    def level(self, l: int, which: str) -> np.ndarray:
        nx, ny, nz = self.levels[l]["dims"]
        out = np.empty((nz, ny, nx), np.float32)
        self._check(self._lib.fire_sim_level_io(self._h, l, 0 if which == "p" else 1, _ptr(out), out.nbytes, 0), "level")
        return out

    def set_level(self, l: int, which: str, arr: np.ndarray):
        a = np.ascontiguousarray(arr, np.float32)
        self._check(self._lib.fire_sim_level_io(self._h, l, 0 if which == "p" else 1, _ptr(a), a.nbytes, 1), "set_level")

    def profile(self, enable: bool = True):
        self._check(self._lib.fire_sim_profile(self._h, int(enable)), "profile")

    def stage_times(self) -> Dict[str, float]:
        ms = np.zeros(8, np.float32)
        self._check(self._lib.fire_sim_stage_times(self._h, _ptr(ms), 8), "stage_times")
        return {k: float(ms[v]) for k, v in STAGES.items()}

    def residual(self, stream=None) -> float:
        r = ctypes.c_double()
        self._check(self._lib.fire_sim_residual(self._h, ctypes.byref(r), _stream_handle(stream)), "residual")
        return r.value

    # ---- diagnostics (FIRE.stats / FIRE.profile) ----
    def stats(self, name: str = "S", stream=None):
        out = np.zeros(16, np.float64)
        self._check(self._lib.fire_sim_stats(self._h, FIELDS[name], _ptr(out), _stream_handle(stream)), "stats")
        return [{"min": out[4 * c], "max": out[4 * c + 1], "mean": out[4 * c + 2], "bad": int(out[4 * c + 3])}
                for c in range(4)]

    def hrr(self, stream=None) -> float:
        q = ctypes.c_double()
        self._check(self._lib.fire_sim_hrr(self._h, ctypes.byref(q), _stream_handle(stream)), "hrr")
        return q.value

    def set_step_stats(self, enable: bool = True):
        """Per-step diagnostics: each step's graph forms stats_async's values beside the pressure solve."""
        self._check(self._lib.fire_sim_set_step_stats(self._h, int(bool(enable))), "set_step_stats")

    def stats_async(self, out_ptr: int, stream=None):
        """Queues S stats + heat release into a pinned host buffer of 17 doubles (no wait)."""
        self._check(self._lib.fire_sim_stats_async(self._h, ctypes.c_void_p(out_ptr), _stream_handle(stream)), "stats_async")

    def height_profile(self, stream=None) -> np.ndarray:
        """Rows (h, Tc, Tmax, soot, fuel, hot) for y rows 0, 4, 8, ... (src/main.js:322-340), unrounded."""
        n = (self.res[1] + 3) // 4
        out = np.zeros((n, 6), np.float64)
        got = ctypes.c_int()
        self._check(self._lib.fire_sim_height_profile(self._h, _ptr(out), n, ctypes.byref(got), _stream_handle(stream)),
                    "height_profile")
        return out[:got.value]

    def fire_profile(self, stream=None) -> dict:
        """FIRE.profile (src/main.js:320-353): heat release and the height profile, rounded for display as the
        reference does (`+x.toFixed(n)` and `Math.round`)."""
        rows = [{"h": js_to_fixed(r[0], 2), "Tc": js_round(r[1]), "Tmax": js_round(r[2]), "soot": js_to_fixed(r[3], 2),
                 "fuel": js_to_fixed(r[4], 2), "hotCells": int(r[5])} for r in self.height_profile(stream)]
        return {"Q_kW": js_to_fixed(self.hrr(stream), 1), "rows": rows}


def js_to_fixed(x: float, digits: int) -> float:
    """JavaScript's `+x.toFixed(digits)`: the decimal nearest the exact binary value of x, a tie going to the
    larger magnitude (Number.prototype.toFixed, ECMA-262), read back as a double."""
    from decimal import Decimal, ROUND_HALF_UP
    return float(Decimal(x).quantize(Decimal(1).scaleb(-digits), rounding=ROUND_HALF_UP))


def js_round(x: float) -> int:
    """JavaScript's `Math.round`: the nearest integer, a tie going toward +infinity (no x + 0.5 rounding step)."""
    r = float(np.floor(x))
    return int(r + 1.0 if x - r >= 0.5 else r)


# ---------------------------------------------------------------------------------------------------
SPARK_FIELDS = ("dt", "time", "frame", "count", "nBase", "nBurst", "burstX", "burstY", "burstZ", "burstSpeed", "burstRadius",
                "ox", "oy", "oz", "sx", "sy", "sz", "turb", "lifeK", "bedRadius", "seed", "sizeK", "upK",
                "burstFan", "burstSize", "aimX", "aimZ")   # src/sparks.js:9-13


class Sparks:
    """Sparks carried by `sim`'s velocity field (src/sparks.js: Sparks)."""

    def __init__(self, sim: "FireSim", count: int = 8192):
        self._lib = load_library()
        self.sim = sim
        self.count = int(count)
        h = ctypes.c_void_p()
        rc = self._lib.fire_sparks_create(sim._h, self.count, ctypes.byref(h))
        if rc:
            raise FireError(rc, "fire_sparks_create")
        self._h = h

    def _check(self, rc: int, what: str):
        if rc:
            raise FireError(rc, what)

    def close(self):
        if self._h is not None:
            self._lib.fire_sparks_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        self._check(self._lib.fire_sparks_reset(self._h), "fire_sparks_reset")

    def burst(self, n: int = 60, pos=(0.0, 0.1, 0.0), speed: float = 3.0, radius: float = 0.05, dur: float = 0.12,
              fan: float = 0.6, size: float = 1.3, aim=None):
        p = np.ascontiguousarray(pos, np.float32)
        a = np.ascontiguousarray(aim, np.float32) if aim is not None else None
        self._check(self._lib.fire_sparks_burst(self._h, int(n), _ptr(p), speed, radius, dur, fan, size,
                                                _ptr(a) if a is not None else None), "fire_sparks_burst")

    def set(self, rate: float = 3.0, turb: float = 1.0, lifeK: float = 1.0, sizeK: float = 1.0, upK: float = 1.0):
        self._check(self._lib.fire_sparks_set(self._h, rate, turb, lifeK, sizeK, upK), "fire_sparks_set")

    def step(self, dt: float, stream=None):
        self._check(self._lib.fire_sparks_step(self._h, float(dt), _stream_handle(stream)), "fire_sparks_step")

    def peek(self, dt: float) -> np.ndarray:
        out = np.zeros(27, np.float32)
        self._check(self._lib.fire_sparks_peek(self._h, float(dt), _ptr(out)), "fire_sparks_peek")
        return out

    def download(self) -> np.ndarray:
        out = np.zeros((self.count, 16), np.float32)
        self._check(self._lib.fire_sparks_io(self._h, _ptr(out), out.nbytes, 0), "fire_sparks_io")
        return out

    def upload(self, arr: np.ndarray):
        a = np.ascontiguousarray(arr, np.float32)
        self._check(self._lib.fire_sparks_io(self._h, _ptr(a), a.nbytes, 1), "fire_sparks_io")


# ---------------------------------------------------------------------------------------------------
def blackbody_lut(n: int = 1024, tmin: float = 400.0, tmax: float = 3000.0, white_balance: float = 5000.0) -> np.ndarray:
    """blackbodyLUT (src/blackbody.js:78-93) as (2, n, 4): rows blackbody and soot, (r, g, b, Y)."""
    out = np.zeros((2, n, 4), np.float32)
    rc = load_library().fire_blackbody_lut(n, tmin, tmax, white_balance, _ptr(out))
    if rc:
        raise FireError(rc, "fire_blackbody_lut")
    return out


class Volume:
    """The renderer's fire passes (lights, prefilter, ray march) into a vw x vh image of `sim`."""

    def __init__(self, sim: "FireSim", width: int = 540, height: int = 960, vol_scale: float = 0.5, white_balance: float = 5000.0):
        self._lib = load_library()
        self.sim = sim
        h = ctypes.c_void_p()
        rc = self._lib.fire_volume_create(sim._h, int(width), int(height), float(vol_scale), float(white_balance), ctypes.byref(h))
        if rc:
            raise FireError(rc, "fire_volume_create")
        self._h = h
        a, b = ctypes.c_int(), ctypes.c_int()
        self._lib.fire_volume_size(self._h, ctypes.byref(a), ctypes.byref(b))
        self.vw, self.vh = a.value, b.value

    def _check(self, rc: int, what: str):
        if rc:
            raise FireError(rc, what)

    def close(self):
        if self._h is not None:
            self._lib.fire_volume_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: Dict[str, float]):
        names = (ctypes.c_char_p * len(params))(*[k.encode() for k in params])
        vals = np.array(list(params.values()), np.float32)
        self._check(self._lib.fire_volume_set_params(self._h, names, _ptr(vals), len(params)), "fire_volume_set_params")

    def set_camera(self, pos, target, fov: float = 40.0, jitter=(0.0, 0.0)):
        p, t = np.asarray(pos, np.float64), np.asarray(target, np.float64)
        self._check(self._lib.fire_volume_set_camera(self._h, _ptr(p), _ptr(t), float(fov), float(jitter[0]), float(jitter[1])),
                    "fire_volume_set_camera")

    def uniforms(self, time: float, frame: int) -> np.ndarray:
        out = np.zeros(64, np.float32)
        n = self._lib.fire_volume_uniforms(self._h, float(time), int(frame), _ptr(out), 64)
        if n < 0:
            raise FireError(n, "fire_volume_uniforms")
        return out[:n]

    def render(self, time: float, frame: int, stream=None):
        self._check(self._lib.fire_volume_render(self._h, float(time), int(frame), _stream_handle(stream)), "fire_volume_render")

    def _get(self, which: int, shape) -> np.ndarray:
        out = np.zeros(shape, np.float32)
        self._check(self._lib.fire_volume_download(self._h, which, _ptr(out), out.nbytes), "fire_volume_download")
        return out

    def image(self) -> np.ndarray:
        return self._get(0, (self.vh, self.vw, 4))

    def aux(self) -> np.ndarray:
        return self._get(1, (self.vh, self.vw, 2))

    def lights(self) -> np.ndarray:
        return self._get(2, (8, 8))


# ---------------------------------------------------------------------------------------------------
# Discrete adjoint of the step over checkpointed rollouts (reverse-mode derivatives; no counterpart in
# the reference).
ADJ_BUFFERS = {"vel": 0, "S": 1, "S2": 2, "velX": 3, "SX": 4, "S2X": 5, "velY": 6, "SY": 7, "S2Y": 8,
               "F": 9, "W": 10, "G": 11, "p": 12, "b": 13}


class Adjoint:
    """Reverse-mode derivatives of `n_steps` steps of `sim`, keeping the state every `checkpoint_every`
    steps.  forward() runs the rollout from the simulation's current state (leaving it in the final state);
    loss() or seed() sets the final-state cotangents; backward() leaves the initial-state cotangents in
    get("vel" / "S" / "S2") and the spot-flux gradients in grad_spots()."""

    def __init__(self, sim: "FireSim", n_steps: int, checkpoint_every: int = 10):
        self._lib = load_library()
        self.sim = sim
        self.n_steps = int(n_steps)
        h = ctypes.c_void_p()
        rc = self._lib.fire_adjoint_create(sim._h, self.n_steps, int(checkpoint_every), ctypes.byref(h))
        if rc:
            raise FireError(rc, "fire_adjoint_create")
        self._h = h

    def _check(self, rc: int, what: str):
        self.sim._check(rc, what)

    def close(self):
        if getattr(self, "_h", None) is not None:
            self._lib.fire_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, dt: float, stream=None):
        self._check(self._lib.fire_adjoint_forward(self._h, float(dt), _stream_handle(stream)), "fire_adjoint_forward")

    def loss(self, target_S: np.ndarray) -> float:
        t = np.ascontiguousarray(target_S, np.float32)
        out = ctypes.c_double()
        self._check(self._lib.fire_adjoint_loss(self._h, _ptr(t), ctypes.byref(out)), "fire_adjoint_loss")
        return out.value

    def seed(self, vel=None, S=None, S2=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (vel, S, S2)]
        self._check(self._lib.fire_adjoint_seed(self._h, *[None if a is None else _ptr(a) for a in arrs]), "fire_adjoint_seed")

    def backward(self, stream=None):
        self._check(self._lib.fire_adjoint_backward(self._h, _stream_handle(stream)), "fire_adjoint_backward")

    def grad_spots(self, n: int) -> np.ndarray:
        out = np.zeros(int(n), np.float64)
        self._check(self._lib.fire_adjoint_grad_spots(self._h, _ptr(out), int(n)), "fire_adjoint_grad_spots")
        return out

    def _shape(self, name: str):
        nx, ny, nz = self.sim.res
        return (nz, ny, nx) + (() if ADJ_BUFFERS[name] >= 12 else (4,))

    def get(self, name: str) -> np.ndarray:
        out = np.zeros(self._shape(name), np.float32)
        self._check(self._lib.fire_adjoint_io(self._h, ADJ_BUFFERS[name], _ptr(out), out.nbytes, 0), f"adjoint get {name}")
        return out

    def put(self, name: str, arr: np.ndarray):
        shape = self._shape(name)
        a = np.ascontiguousarray(arr, np.float32)
        if a.size != int(np.prod(shape)):
            raise FireError(1, f"adjoint put {name}: expected shape {shape}")
        a = a.reshape(shape)
        self._check(self._lib.fire_adjoint_io(self._h, ADJ_BUFFERS[name], _ptr(a), a.nbytes, 1), f"adjoint put {name}")

    def clear(self):
        self._check(self._lib.fire_adjoint_clear(self._h), "fire_adjoint_clear")

    def stage(self, name: str, dt: float, arg: int = 0, stream=None):
        self._check(self._lib.fire_adjoint_stage(self._h, STAGES[name], float(dt), int(arg), _stream_handle(stream)),
                    f"fire_adjoint_stage {name}")

    def timing(self):
        f, b = ctypes.c_float(), ctypes.c_float()
        self._check(self._lib.fire_adjoint_timing(self._h, ctypes.byref(f), ctypes.byref(b)), "fire_adjoint_timing")
        return f.value, b.value


def rollout_function():
    """A torch.autograd.Function over an Adjoint:  FireRollout.apply(adj, dt, spots, vel0, S0, S2_0, fluxes)
    sets the simulation's state and spot fluxes (spots: (n, 5) records whose flux column is replaced by
    `fluxes`), runs the rollout and returns the final (vel, S, S2); its backward runs the reverse sweep and
    returns the gradients of vel0, S0, S2_0 and the fluxes.  Tensors live on the host (float32 fields,
    float64 fluxes); the rollout itself runs on the device through the C ABI."""
    import torch

    class FireRollout(torch.autograd.Function):
        @staticmethod
        def forward(ctx, adj, dt, spots, vel0, S0, S2_0, fluxes):
            sim = adj.sim
            sp = np.array(spots, np.float32).reshape(-1, 5)
            sp[:, 4] = fluxes.detach().cpu().numpy().astype(np.float32)
            sim.set_spots(sp)
            for name, a in (("vel", vel0), ("S", S0), ("S2", S2_0)):
                sim.upload(name, a.detach().cpu().numpy())
            adj.forward(dt)
            sim.sync()
            ctx.adj, ctx.n = adj, len(sp)
            return tuple(torch.from_numpy(sim.download(n).astype(np.float32)) for n in ("vel", "S", "S2"))

        @staticmethod
        def backward(ctx, gvel, gS, gS2):
            adj = ctx.adj
            adj.seed(*[None if g is None else g.detach().cpu().numpy() for g in (gvel, gS, gS2)])
            adj.backward()
            grads = [torch.from_numpy(adj.get(n)) for n in ("vel", "S", "S2")]
            return (None, None, None, *grads, torch.from_numpy(adj.grad_spots(ctx.n)))

    return FireRollout


# ---------------------------------------------------------------------------------------------------
# The cinematic's timeline (src/timeline.js) and its capture-mode driver (src/main.js:128-160).
EVENT_TYPES = {0: "pop", 1: "crackle-burst", 2: "log-shift", 3: "gust", 4: "ignite"}


class FireTimelineEvent(ctypes.Structure):
    _fields_ = [("t", ctypes.c_double), ("type", ctypes.c_int), ("strength", ctypes.c_double), ("pos", ctypes.c_double * 3),
                ("has_aim", ctypes.c_int), ("aim", ctypes.c_double * 3), ("log", ctypes.c_int), ("dur", ctypes.c_double)]


def timeline_events():
    L = load_library()
    n = L.fire_timeline_event_count()
    arr = (FireTimelineEvent * n)()
    L.fire_timeline_events(arr, n)
    return [{"t": e.t, "type": EVENT_TYPES[e.type], "strength": e.strength, "pos": tuple(e.pos),
             "aim": tuple(e.aim) if e.has_aim else None, "log": e.log, "dur": e.dur} for e in arr]


def timeline_sim_at(t: float) -> Dict[str, float]:
    out = np.zeros(7, np.float64)
    load_library().fire_timeline_sim_at(float(t), _ptr(out))
    return dict(zip(("intensity", "burstAmt", "burstX", "burstY", "burstZ", "windX", "windZ"), map(float, out)))


def timeline_intensity_at(t: float) -> float:
    return float(load_library().fire_timeline_intensity_at(float(t)))


def timeline_log_offsets_at(t: float):
    i, s, a, b, c = ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    if not load_library().fire_timeline_log_offsets_at(float(t), ctypes.byref(i), ctypes.byref(s), ctypes.byref(a),
                                                       ctypes.byref(b), ctypes.byref(c)):
        return None
    return {"index": i.value, "s": s.value, "footOut": a.value, "topDrop": b.value, "topOut": c.value}


def timeline_camera_at(t: float):
    pos, tgt, fov = np.zeros(3), np.zeros(3), ctypes.c_double()
    load_library().fire_timeline_camera_at(float(t), _ptr(pos), _ptr(tgt), ctypes.byref(fov))
    return {"pos": tuple(pos), "target": tuple(tgt), "fov": fov.value}


def timeline_lens_at(t: float):
    f, a, m, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    load_library().fire_timeline_lens_at(float(t), ctypes.byref(f), ctypes.byref(a), ctypes.byref(m), ctypes.byref(n))
    return {"focus": f.value, "aperture": a.value, "fmm": m.value, "N": n.value}


class Timeline:
    """capStep driver: `step(j)` sets sim params and log offsets for t = j / (30 n), throws the event bursts
    and steps the simulation (and the sparks, if given) by 1 / (30 n)."""

    def __init__(self, base_logs: np.ndarray, steps_per_frame: int = 8):
        self._lib = load_library()
        lg = np.ascontiguousarray(base_logs, np.float32).reshape(-1)
        h = ctypes.c_void_p()
        rc = self._lib.fire_timeline_create(_ptr(lg) if lg.size else None, lg.size // 8, int(steps_per_frame), ctypes.byref(h))
        if rc:
            raise FireError(rc, "fire_timeline_create")
        self._h = h
        self.dt = float(self._lib.fire_timeline_step_dt(self._h))

    def time(self, j: int) -> float:
        return float(self._lib.fire_timeline_step_time(self._h, int(j)))

    def step(self, sim: "FireSim", j: int, sparks: Optional["Sparks"] = None, stream=None):
        rc = self._lib.fire_timeline_step(self._h, sim._h, sparks._h if sparks is not None else None, int(j), _stream_handle(stream))
        if rc:
            raise FireError(rc, "fire_timeline_step")

    def close(self):
        if self._h is not None:
            self._lib.fire_timeline_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------------------------------
class Ensemble:
    """Independent simulations of possibly different grids stepped together (one launch per stage over all
    members).  `members[i]` is a FireSim view for configuring and reading member i; step with `step`."""

    def __init__(self, configs: Sequence[dict], vcycles: int = 4, device: int = 0, noise_seed: int = 1):
        self._lib = load_library()
        self._h = None
        n = len(configs)
        arr = (FireConfig * n)()
        for i, c in enumerate(configs):
            arr[i].res[:] = [int(r) for r in c["res"]]
            arr[i].size[:] = [float(s) for s in c["size"]]
            arr[i].vcycles = int(vcycles)
            arr[i].device = int(device)
            arr[i].noise_seed = int(noise_seed)
            arr[i].mg_max_cycles = 0
            arr[i].mg_tol = 0.0
        h = ctypes.c_void_p()
        rc = self._lib.fire_ensemble_create(arr, n, ctypes.byref(h))
        if rc:
            raise FireError(rc, "fire_ensemble_create")
        self._h = h
        self.members = []
        for i in range(n):
            s = ctypes.c_void_p()
            self._check(self._lib.fire_ensemble_sim(self._h, i, ctypes.byref(s)), "fire_ensemble_sim")
            self.members.append(FireSim._borrow(s))

    def _check(self, rc: int, what: str):
        if rc:
            msg = self._lib.fire_ensemble_last_error(self._h) if self._h else b""
            raise FireError(rc, f"{what}: {msg.decode() if msg else ''}")

    def step(self, dt: float, n: int = 1, stream=None):
        self._check(self._lib.fire_ensemble_step(self._h, float(dt), int(n), _stream_handle(stream)), "fire_ensemble_step")

    def sync(self):
        self._check(self._lib.fire_ensemble_sync(self._h), "fire_ensemble_sync")

    # stage order of the tile choices: adv1, adv2, forces, div, project
    def set_autotune(self, at_step: int):
        """Tune the tiles on step number `at_step` from now on the ensemble's count (-1: never)."""
        self._check(self._lib.fire_ensemble_set_autotune(self._h, int(at_step)), "fire_ensemble_set_autotune")

    def set_tiles(self, tiles: Sequence[int]):
        a = np.ascontiguousarray(tiles, np.int32)
        self._check(self._lib.fire_ensemble_set_tiles(self._h, _ptr(a)), "fire_ensemble_set_tiles")

    def tiles(self):
        """(chosen tile per stage, measured mean launch ms per stage and candidate (5 x 4)), or None before
        the tuning step."""
        a = np.zeros(5, np.int32)
        ms = np.zeros((5, 4), np.float32)
        rc = self._lib.fire_ensemble_tiles(self._h, _ptr(a), _ptr(ms))
        if rc == 6:
            return None
        self._check(rc, "fire_ensemble_tiles")
        return a, ms

    def close(self):
        if self._h is not None:
            for m in self.members:
                m._h = None
            self._lib.fire_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------------------------------
# Standalone pressure Poisson solver (the step's multigrid, src/sim.js:415-495, 576-599, iterated to a
# tolerance; plain FP32 or FP16/BF16-storage iterative refinement).
PRECISIONS = {"fp32": 0, "fp16": 1, "bf16": 2, "ir32": 3}


class FirePoissonResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("rel_residual", ctypes.c_double),
                ("rel_residual_initial", ctypes.c_double), ("b_norm", ctypes.c_double)]


def _dev_ptr(a) -> int:
    """Device address of a torch tensor (or an int address)."""
    return int(a) if isinstance(a, int) else int(a.data_ptr())


def poisson_sources(seed: int, n: int, res) -> np.ndarray:
    """The (centre x, y, z, sigma, amplitude) rows of fire_poisson_make_rhs, cell units."""
    out = np.zeros((max(n, 1), 5), np.float32)
    r = (ctypes.c_int * 3)(*[int(v) for v in res])
    rc = load_library().fire_poisson_sources(seed, n, r, _ptr(out))
    if rc:
        raise FireError(rc, "poisson_sources")
    return out[:n]


class Poisson:
    """Standalone solver for the step's pressure equation on device arrays of res[0]*res[1]*res[2] floats."""

    def __init__(self, res, h: float, precision: str = "fp32", device: int = 0):
        self._lib = load_library()
        self.res = tuple(int(v) for v in res)
        self.h = float(h)
        self.precision = precision
        r = (ctypes.c_int * 3)(*self.res)
        hnd = ctypes.c_void_p()
        rc = self._lib.fire_poisson_create(r, self.h, PRECISIONS[precision], device, ctypes.byref(hnd))
        if rc:
            raise FireError(rc, "fire_poisson_create")
        self._h = hnd

    def close(self):
        if self._h:
            self._lib.fire_poisson_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc:
            raise FireError(rc, what)

    def solve(self, b, x, tol: float = 1e-6, max_iters: int = 50, inner_cycles: int = 1, x_lo=None, stream=None):
        """Queues the solve of A x = b (x, and x_lo if given, hold the initial guess); returns without waiting."""
        lo = ctypes.c_void_p(_dev_ptr(x_lo)) if x_lo is not None else None
        self._check(self._lib.fire_poisson_solve(self._h, ctypes.c_void_p(_dev_ptr(b)), ctypes.c_void_p(_dev_ptr(x)), lo, float(tol),
                                                 int(max_iters), int(inner_cycles), _stream_handle(stream)), "fire_poisson_solve")

    def result(self) -> Dict[str, float]:
        r = FirePoissonResult()
        self._check(self._lib.fire_poisson_result(self._h, ctypes.byref(r)), "fire_poisson_result")
        return {"iterations": r.iterations, "rel_residual": r.rel_residual,
                "rel_residual_initial": r.rel_residual_initial, "b_norm": r.b_norm}

    def residual(self, b, x, x_lo=None) -> float:
        v = ctypes.c_double()
        lo = ctypes.c_void_p(_dev_ptr(x_lo)) if x_lo is not None else None
        self._check(self._lib.fire_poisson_residual(self._h, ctypes.c_void_p(_dev_ptr(b)), ctypes.c_void_p(_dev_ptr(x)), lo,
                                                    ctypes.byref(v)), "fire_poisson_residual")
        return v.value

    def set_study(self, coarse_sweeps: int):
        """FP32 form: switch to the V-cycle variant of the reference's multigrid convergence studies
        (research/webgpu-bench/poisson.mjs, wgsl/mg.wgsl) with `coarse_sweeps` coarsest-level sweeps."""
        self._check(self._lib.fire_poisson_set_study(self._h, int(coarse_sweeps)), "fire_poisson_set_study")

    def make_rhs(self, b, seed: int = 3, n_sources: int = 32, noise: float = 1e-3, stream=None):
        self._check(self._lib.fire_poisson_make_rhs(self._h, ctypes.c_void_p(_dev_ptr(b)), seed, n_sources, float(noise),
                                                    _stream_handle(stream)), "fire_poisson_make_rhs")
