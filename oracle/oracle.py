"""ctypes wrapper over the CPU oracle (libfire_oracle.so).  TEST INFRASTRUCTURE ONLY.

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline and reference legs of ``bench.py``
import this module; it is the checker for the CUDA product path, never part of it.  The oracle restates the
reference WGSL kernels of src/sim.js (see fire_oracle.cpp for the per-kernel citations).  Its multigrid is
pinned to the reference's recorded convergence studies; advection, the source terms and projection are
parity unpinned by the reference (no golden vectors exist and its WGSL cannot run here) and are pinned only
by the restatement and the independent numpy restatements in tests/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libfire_oracle.so"

# Field ids shared with the CUDA library (src/sim.js:72-76 texture names)
FIELDS = {"vel": 0, "velX": 1, "velY": 2, "S": 3, "SX": 4, "SY": 5, "S2": 6, "S2X": 7, "S2Y": 8,
          "vort": 9, "geo": 10}
STAGES = {"geo": 0, "adv1": 1, "adv2": 2, "curl": 3, "forces": 4, "div": 5, "vcycle": 6, "project": 7}


def build(force: bool = False) -> Path:
    """Compile the oracle shared library with its Makefile (g++ -fopenmp)."""
    src = HERE / "fire_oracle.cpp"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        vp, ip, fp, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
        sigs = {
            "orc_num_threads": (ip, []), "orc_set_threads": (None, [ip]),
            "orc_noise_table": (None, [ip, ip, vp]), "orc_curl_table": (None, [ip, vp, vp]),
            "orc_f32_to_f16": (ctypes.c_uint16, [fp]), "orc_f16_to_f32": (fp, [ctypes.c_uint16]),
            "orc_hash3f": (None, [ip, ip, ip, vp]), "orc_pcg": (ctypes.c_uint32, [ctypes.c_uint32]),
            "orc_rand2": (fp, [ctypes.c_uint32, ctypes.c_uint32]),
            "orc_build_campfire": (None, [ctypes.c_uint32, vp]),
            "orc_create": (vp, [ip, ip, ip, dp, ip]), "orc_destroy": (None, [vp]),
            "orc_num_levels": (ip, [vp]), "orc_level_info": (None, [vp, ip, vp, vp]),
            "orc_coarse_iters": (ip, [vp]), "orc_set_params": (None, [vp, vp]), "orc_set_ext": (None, [vp, vp]),
            "orc_ext_count": (ip, []), "orc_set_logs": (None, [vp, vp, ip]),
            "orc_set_tables": (None, [vp, ip, vp, vp]),
            "orc_get_field": (ip, [vp, ip, vp, ip]), "orc_set_field": (ip, [vp, ip, vp, ip]),
            "orc_get_level": (ip, [vp, ip, ip, vp, ip]), "orc_set_level": (ip, [vp, ip, ip, vp, ip]),
            "orc_stage": (None, [vp, ip]), "orc_mg_smooth": (None, [vp, ip, ip]),
            "orc_mg_restrict": (None, [vp, ip]), "orc_mg_prolong": (None, [vp, ip]),
            "orc_mg_vcycle": (None, [vp, ip, ip]), "orc_residual": (None, [vp, vp, vp]),
            "orc_step": (ip, [vp, ip, ip, dp]), "orc_reset": (None, [vp]),
            "orc_poisson_study": (dp, [ip, ip, ip, dp, ip, ip, ip, ip, vp]),
            "orc_poisson_rhs": (None, [ip, vp]),
            "orc_pressure_apply": (None, [ip, ip, ip, dp, vp, vp]),
            "orc_pressure_rel_residual": (dp, [ip, ip, ip, dp, vp, vp]),
            "orc_pressure_cg": (ip, [ip, ip, ip, dp, vp, vp, dp, ip, vp]),
            "orc_sparks_step": (None, [vp, ip, vp, vp, ip, ip, ip, vp, ip]),
            "orc_volume_lights": (None, [vp, vp, ip, ip, ip, vp, vp, vp]),
            "orc_volume_render": (None, [vp, vp, vp, ip, ip, ip, vp, ip, vp, vp, vp, vp]),
            "orc_set_modes": (None, [vp, dp, ip, ip]), "orc_set_coarse_iters": (None, [vp, ip]),
            "orc_sim_defaults": (None, [vp]), "orc_set_flux64": (None, [vp, vp, ip]),
            "orc_make_spots": (None, [ctypes.c_uint32, ip, fp, fp, fp, fp, vp]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def noise_table(N: int = 128, seed: int = 1) -> np.ndarray:
    out = np.empty((N, N, N, 4), np.float32)
    lib().orc_noise_table(N, seed, _ptr(out))
    return out


def curl_table(noise: np.ndarray) -> np.ndarray:
    N = noise.shape[0]
    noise = np.ascontiguousarray(noise, np.float32)
    out = np.empty_like(noise)
    lib().orc_curl_table(N, _ptr(noise), _ptr(out))
    return out


def build_campfire(seed: int = 7) -> np.ndarray:
    out = np.zeros(128, np.float32)
    lib().orc_build_campfire(seed, _ptr(out))
    return out


def poisson_rhs(N: int) -> np.ndarray:
    """The convergence study's right-hand side (research/webgpu-bench/poisson.mjs:78-92), (N, N, N) float32."""
    out = np.zeros(N * N * N, np.float32)
    lib().orc_poisson_rhs(int(N), _ptr(out))
    return out.reshape(N, N, N)


def sim_defaults() -> np.ndarray:
    """SIM_DEFAULTS (src/sim.js:25-44) as the 64-float block in SIM_FIELDS order (simulation-owned slots 0)."""
    out = np.zeros(64, np.float32)
    lib().orc_sim_defaults(_ptr(out))
    return out


def make_spots(seed: int, n: int, flux_lo: float = 1.0, flux_hi: float = 4.0, sigma: float = 0.02,
               radius: float = 0.15) -> np.ndarray:
    """The synthetic workloads' seeded floor spots, (n, 5) = (x, y, z, sigma, flux g/s)."""
    out = np.zeros((max(n, 1), 5), np.float32)
    lib().orc_make_spots(int(seed) & 0xFFFFFFFF, int(n), float(flux_lo), float(flux_hi), float(sigma), float(radius), _ptr(out))
    return out[:n]


def poisson_study(N: int, face: bool, mode: int, omega: float = 1.0, pre: int = 2, post: int = 2,
                  coarse: int = 30, cycles: int = 8):
    hist = np.zeros(max(cycles, 6), np.float64)
    r0 = lib().orc_poisson_study(N, int(face), mode, omega, pre, post, coarse, cycles, _ptr(hist))
    n = 6 if mode in (0, 1) else cycles
    return r0, hist[:n]


def sparks_step(sparks: np.ndarray, uniforms: np.ndarray, vel: np.ndarray, curl: np.ndarray) -> np.ndarray:
    """One spark update (src/sparks.js:55-142) of a (count, 16) array; vel is (nz, ny, nx, 4), curl (N, N, N, 4)."""
    s = np.ascontiguousarray(sparks, np.float32).copy()
    U = np.ascontiguousarray(uniforms, np.float32)
    v = np.ascontiguousarray(vel, np.float32)
    c = np.ascontiguousarray(curl, np.float32)
    nz, ny, nx = v.shape[:3]
    lib().orc_sparks_step(_ptr(s), s.shape[0], _ptr(U), _ptr(v), nx, ny, nz, _ptr(c), c.shape[0])
    return s


def volume_lights(uniforms, S, lut, lstate):
    """pLights (src/renderer.js:104-165): returns (lights (8, 8), new lstate (24, 4))."""
    U = np.ascontiguousarray(uniforms, np.float32)
    s = np.ascontiguousarray(S, np.float32)
    L = np.ascontiguousarray(lut, np.float32)
    st = np.ascontiguousarray(lstate, np.float32).copy()
    out = np.zeros((8, 8), np.float32)
    nz, ny, nx = s.shape[:3]
    lib().orc_volume_lights(_ptr(U), _ptr(s), nx, ny, nz, _ptr(L), _ptr(st), _ptr(out))
    return out, st


def volume_render(uniforms, S, S2, curl, lut, lights):
    """pVolume (src/renderer.js:194-326) without a depth buffer: returns (image (vh, vw, 4), aux (vh, vw, 2))."""
    U = np.ascontiguousarray(uniforms, np.float32)
    s, s2 = np.ascontiguousarray(S, np.float32), np.ascontiguousarray(S2, np.float32)
    c, L, li = np.ascontiguousarray(curl, np.float32), np.ascontiguousarray(lut, np.float32), np.ascontiguousarray(lights, np.float32)
    vw, vh = int(U[2]), int(U[3])
    img, aux = np.zeros((vh, vw, 4), np.float32), np.zeros((vh, vw, 2), np.float32)
    nz, ny, nx = s.shape[:3]
    lib().orc_volume_render(_ptr(U), _ptr(s), _ptr(s2), nx, ny, nz, _ptr(c), c.shape[0], _ptr(L), _ptr(li), _ptr(img), _ptr(aux))
    return img, aux


def pressure_apply(x: np.ndarray, h: float) -> np.ndarray:
    """A x in FP64 (the multigrid's operator with its ghost rules); x indexed [z, y, x]."""
    x = np.ascontiguousarray(x, np.float64)
    nz, ny, nx = x.shape
    out = np.empty_like(x)
    lib().orc_pressure_apply(nx, ny, nz, float(h), _ptr(x), _ptr(out))
    return out


def pressure_rel_residual(b: np.ndarray, x: np.ndarray, h: float) -> float:
    """||b - A x|| / ||b|| in FP64 of FP32 arrays indexed [z, y, x]."""
    b = np.ascontiguousarray(b, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    nz, ny, nx = b.shape
    return float(lib().orc_pressure_rel_residual(nx, ny, nz, float(h), _ptr(b), _ptr(x)))


def pressure_cg(b: np.ndarray, h: float, tol: float = 1e-12, maxit: int = 100000):
    """FP64 conjugate-gradient solution of A x = b; returns (x, iterations, relative residual)."""
    b = np.ascontiguousarray(b, np.float64)
    nz, ny, nx = b.shape
    x = np.zeros_like(b)
    rel = np.zeros(1, np.float64)
    it = lib().orc_pressure_cg(nx, ny, nz, float(h), _ptr(b), _ptr(x), float(tol), int(maxit), _ptr(rel))
    return x, int(it), float(rel[0])


class OracleSim:
    """CPU restatement of FireSim (src/sim.js:48-649); dbl=True runs in FP64."""

    def __init__(self, res, dx: float, dbl: bool = False):
        self.res = tuple(int(r) for r in res)
        self.dbl = bool(dbl)
        self.h = lib().orc_create(self.res[0], self.res[1], self.res[2], float(dx), int(dbl))
        self.nlevels = lib().orc_num_levels(self.h)
        self.levels = []
        for l in range(self.nlevels):
            d = np.zeros(3, np.int32)
            hh = np.zeros(1, np.float64)
            lib().orc_level_info(self.h, l, _ptr(d), _ptr(hh))
            self.levels.append((tuple(int(v) for v in d), float(hh[0])))
        self.coarse_iters = lib().orc_coarse_iters(self.h)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    @property
    def cells(self):
        return self.res[0] * self.res[1] * self.res[2]

    def set_params(self, p64: np.ndarray):
        p = np.ascontiguousarray(p64, np.float32)
        assert p.size == 64
        lib().orc_set_params(self.h, _ptr(p))

    def set_ext(self, ext: np.ndarray):
        e = np.ascontiguousarray(ext, np.float32)
        assert e.size == lib().orc_ext_count()
        lib().orc_set_ext(self.h, _ptr(e))

    def set_logs(self, logs: np.ndarray):
        lg = np.ascontiguousarray(logs, np.float32)
        lib().orc_set_logs(self.h, _ptr(lg), lg.size // 8)

    def set_tables(self, noise: np.ndarray, curl: np.ndarray):
        n = np.ascontiguousarray(noise, np.float32)
        c = np.ascontiguousarray(curl, np.float32)
        lib().orc_set_tables(self.h, n.shape[0], _ptr(n), _ptr(c))

    def _shape(self):
        return (self.res[2], self.res[1], self.res[0], 4)

    def get(self, name: str, dtype=np.float32) -> np.ndarray:
        out = np.empty(self._shape(), dtype)
        assert lib().orc_get_field(self.h, FIELDS[name], _ptr(out), int(dtype == np.float64)) == 0
        return out

    def put(self, name: str, arr: np.ndarray):
        a = np.ascontiguousarray(arr)
        dbl = a.dtype == np.float64
        if not dbl:
            a = np.ascontiguousarray(a, np.float32)
        assert a.size == self.cells * 4
        assert lib().orc_set_field(self.h, FIELDS[name], _ptr(a), int(dbl)) == 0

    def get_level(self, l: int, which: str, dtype=np.float32) -> np.ndarray:
        (nx, ny, nz), _ = self.levels[l]
        out = np.empty((nz, ny, nx), dtype)
        lib().orc_get_level(self.h, l, 0 if which == "p" else 1, _ptr(out), int(dtype == np.float64))
        return out

    def put_level(self, l: int, which: str, arr: np.ndarray):
        a = np.ascontiguousarray(arr)
        dbl = a.dtype == np.float64
        if not dbl:
            a = np.ascontiguousarray(a, np.float32)
        lib().orc_set_level(self.h, l, 0 if which == "p" else 1, _ptr(a), int(dbl))

    def stage(self, name: str):
        lib().orc_stage(self.h, STAGES[name])

    def mg_smooth(self, l: int, color: int):
        lib().orc_mg_smooth(self.h, l, color)

    def mg_restrict(self, l: int):
        lib().orc_mg_restrict(self.h, l)

    def mg_prolong(self, l: int):
        lib().orc_mg_prolong(self.h, l)

    def vcycle(self, pre: int = 2, post: int = 2):
        lib().orc_mg_vcycle(self.h, pre, post)

    def residual(self):
        rr = np.zeros(1, np.float64)
        bb = np.zeros(1, np.float64)
        lib().orc_residual(self.h, _ptr(rr), _ptr(bb))
        return float(rr[0]), float(bb[0])

    def step_raw(self, rebuild_geo: bool, vcycles: int, tol: float = 0.0) -> int:
        """One step; vcycles < 0 solves to `tol` relative residual in at most -vcycles cycles (returns cycles run)."""
        return lib().orc_step(self.h, int(rebuild_geo), int(vcycles), float(tol))

    def set_modes(self, omega: float = 1.0, store_half: bool = False, filter_bits: int = 0):
        """omega: over-relaxation of every multigrid sweep (1 = Gauss-Seidel); store_half: round every float4
        field to IEEE half after the stage that writes it (the reference's rgba16float textures); filter_bits:
        fractional bits of the trilinear texture weights (0 = exact)."""
        lib().orc_set_modes(self.h, float(omega), int(bool(store_half)), int(filter_bits))

    def set_flux64(self, flux=None):
        """Spot fluxes (g/s) in double, overriding the extension block's FP32 values (None clears)."""
        f = np.zeros(16, np.float64)
        n = 0 if flux is None else len(flux)
        if n:
            f[:n] = np.asarray(flux, np.float64)
        lib().orc_set_flux64(self.h, _ptr(f), n)

    def set_coarse_iters(self, iters: int):
        lib().orc_set_coarse_iters(self.h, int(iters))
        self.coarse_iters = int(iters)

    def reset(self):
        lib().orc_reset(self.h)
