"""The C ABI library: it loads, exports every entry point include/*.h declares, and its host-only logic
(parameter names/defaults, scene helpers, argument checks) behaves without a GPU."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import fire_sim as F

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(fire_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = F.load_library()
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # and the Python mirror binds exactly the declared set
    assert set(F.EXPORTS) == set(syms)


def test_param_names_and_defaults_follow_sim_fields():
    lib = F.load_library()
    for i, name in enumerate(F.SIM_FIELDS):
        assert lib.fire_param_index(name.encode()) == i
        assert lib.fire_param_name(i).decode() == name
    assert lib.fire_param_index(b"bogus") == -1
    d = F.param_defaults()
    want = dict(fuelSrc=0.13, bedFuel=0.16, srcTemp=0.75, bedTemp=0.82, srcVel=0.25, srcFreq=35.0, srcSpeed=0.06,
                srcThresh=0.0, ignT=550, kMix=30, rs=4.7, heatOut=7700, expansion=0.7, sootForm=25, sootOx=30,
                radCool=0.25, coolRate=3.0, sootDissip=0.4, smokeDissip=0.3, vitDecay=1.5, fuelDissip=0.3,
                buoyancy=26.8, vortEps=8, turbAmp=0.8, turbFreq=1.5, turbRise=1.5, turbEvolve=0.6, windX=0, windZ=0,
                gust=0, intensity=1, velDissip=0.05, bedRadius=0.22, hotR0=0.12, hotR1=0.45, hotY1=0.5, logSrc=1,
                burstX=0, burstY=0, burstZ=0, burstAmt=0, smolder=0.02, sponge=1, visc=0, lamAge=0, anchorFreq=1.6,
                srcFloor=0.25, anchorGain=0.95)
    for k, v in want.items():
        assert d[F.SIM_FIELDS.index(k)] == np.float32(v), k
    assert not d[:12].any() and not d[60:].any()


def test_build_campfire_matches_oracle(oracle_mod):
    for seed in (7, 3, 99):
        np.testing.assert_array_equal(F.build_campfire(seed), oracle_mod.build_campfire(seed))
    assert F.load_library().fire_build_campfire(7, None, 16) != 0


def test_make_spots_deterministic_and_in_disc():
    a = F.make_spots(5, 6, 1.0, 4.0, 0.02, 0.15)
    b = F.make_spots(5, 6, 1.0, 4.0, 0.02, 0.15)
    np.testing.assert_array_equal(a, b)
    r = np.hypot(a[:, 0], a[:, 2])
    assert (r <= 0.15 + 1e-6).all() and (a[:, 1] == 0).all() and (a[:, 3] == np.float32(0.02)).all()
    assert ((a[:, 4] >= 1.0) & (a[:, 4] <= 4.0)).all()
    assert not np.array_equal(a, F.make_spots(6, 6, 1.0, 4.0, 0.02, 0.15))
    with pytest.raises(F.FireError):
        F.make_spots(5, 17)


def test_js_rounding_helpers():
    """FIRE.profile's display rounding: toFixed works on the exact binary value, Math.round ties go up."""
    assert F.js_to_fixed(1.005, 2) == 1.0          # 1.005 is 1.00499999999999989... in binary
    assert F.js_to_fixed(0.125, 2) == 0.13         # an exact tie: the larger n
    assert F.js_to_fixed(-0.125, 2) == -0.13       # toFixed rounds |x| and keeps the sign
    assert F.js_to_fixed(1234.56789, 1) == 1234.6
    assert F.js_round(2.5) == 3 and F.js_round(-2.5) == -2 and F.js_round(1672.49) == 1672
    assert F.js_round(0.49999999999999994) == 0     # floor(x + 0.5) would give 1


def test_host_classes_define_each_method_once():
    """A second definition of a method name silently replaces the first (a FIRE.profile mirror named `profile`
    would hide the per-stage timing switch `profile(enable)` that bench.py uses)."""
    import ast
    import collections
    src = (Path(F.__file__)).read_text()
    for node in ast.walk(ast.parse(src)):
        if isinstance(node, ast.ClassDef):
            names = collections.Counter(n.name for n in node.body if isinstance(n, ast.FunctionDef))
            assert not [k for k, v in names.items() if v > 1], (node.name, names)


def test_argument_checks_without_device():
    lib = F.load_library()
    cfg = F.FireConfig()
    cfg.res[:] = [1, 8, 8]           # res < 2 is rejected before any device call
    cfg.size[:] = [1, 1, 1]
    h = ctypes.c_void_p()
    assert lib.fire_sim_create(ctypes.byref(cfg), None, 0, ctypes.byref(h)) == 1
    cfg.res[:] = [2048, 1024, 1024]  # 2^31 cells: beyond the kernels' 32-bit cell offsets
    assert lib.fire_sim_create(ctypes.byref(cfg), None, 0, ctypes.byref(h)) == 1
    cfg.res[:] = [1, 8, 8]
    assert lib.fire_sim_create(None, None, 0, ctypes.byref(h)) == 1
    for fn in ("fire_sim_step", "fire_sim_reset", "fire_sim_sync"):
        args = {"fire_sim_step": (None, 0.01, 1, None)}.get(fn, (None,))
        assert getattr(lib, fn)(*args) == 1
    assert lib.fire_version().decode().startswith("procedural-fire-gb300")


def test_no_silent_fallback_without_device():
    """Without a GB300 the product path refuses to run (there is no CPU path)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    assert not F.device_ok(0)
    with pytest.raises(F.FireError) as ei:
        F.FireSim(res=(16, 16, 16), size=(0.2, 0.2, 0.2))
    assert ei.value.code == 4


def test_oracle_restates_defaults_and_spots(oracle_mod):
    """The oracle's own SIM_DEFAULTS block and seeded spots (used by bench.py's reference arm, which loads
    no product library) equal the library's."""
    np.testing.assert_array_equal(oracle_mod.sim_defaults(), F.param_defaults())
    for args in [(2, 6, 1.0, 4.0, 0.02, 0.2), (11, 8, 1.0, 4.0, 0.02, 0.12), (1000, 2, 1.0, 4.0, 0.02, 0.18)]:
        np.testing.assert_array_equal(oracle_mod.make_spots(*args), F.make_spots(*args))


def test_reference_arm_inputs_load_no_product_library():
    """bench.py's reference arm builds the workload from the oracle alone: after building its parameter block
    neither the host mirror module nor libfiresim.so is loaded in the process."""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    code = ("import sys; sys.path[:0] = ['oracle']; import bench, oracle; blk = bench.oracle_block(oracle); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'fire_sim' not in sys.modules and 'libfiresim' not in maps, 'product library loaded'; "
            "assert 'libfire_oracle' in maps; print(float(blk[34]), int(blk[64 + 3]))")
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["0.30000001192092896", "6"]
