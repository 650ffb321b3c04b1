"""Kernel-level parity: each CUDA stage against the CPU oracle from identical inputs.

Tables and emitter geometry are compiled without FMA contraction and must be bit-identical.  The hot
stencil kernels keep FMA contraction, so they are held to an FP32 tolerance: |gpu - oracle| <= 1e-4 |oracle|
+ 1e-5 max|oracle| per channel, with at most 0.1 % of cells allowed beyond it (branch flips at
thresholds such as the limiter's floor() or the confinement's |grad w| > 1e-6 test).
"""
import numpy as np
import pytest

import fire_cases as FC
import fire_sim as F

pytestmark = pytest.mark.gpu

RTOL, ATOL, OUTLIERS = 1e-4, 1e-5, 1e-3


@pytest.fixture(scope="module")
def campfire():
    return F.build_campfire(7)


def test_noise_and_curl_tables_bit_exact(tables):
    noise, curl = tables
    sim = F.FireSim(res=(16, 16, 16), size=(0.2, 0.2, 0.2))
    np.testing.assert_array_equal(sim.download("noise").astype(np.float32), noise)
    np.testing.assert_array_equal(sim.download("curl").astype(np.float32), curl)


@pytest.mark.parametrize("variant", ["campfire", "spots_nobed", "hot_radii"])
def test_geo_bit_exact(campfire, variant):
    params = {"hotR0": 0.1, "hotR1": 0.3, "hotY1": 0.4, "bedRadius": 0.18} if variant == "hot_radii" else None
    sim, orc = FC.make_pair(FC.C1, logs=campfire if variant != "spots_nobed" else None,
                            bed_gain=0.0 if variant == "spots_nobed" else None, params=params)
    FC.sync_block(sim, orc, FC.C1["dt"])
    sim.run_stage("geo", FC.C1["dt"])
    orc.stage("geo")
    np.testing.assert_array_equal(sim.download("geo"), orc.get("geo"))


def _stage_case(campfire, stage, params=None, spots=None, seed=3, time=0.37):
    sim, orc = FC.make_pair(FC.C1, logs=campfire, spots=spots, params=params)
    dt = FC.C1["dt"]
    FC.sync_block(sim, orc, dt)
    sim.run_stage("geo", dt)
    orc.stage("geo")
    FC.put_state(sim, orc, FC.random_state(FC.C1["res"], seed))
    blk = FC.sync_block(sim, orc, dt)
    return sim, orc, dt


OUTPUTS = {"adv1": ["velX", "SX", "S2X"], "adv2": ["velY", "SY", "S2Y"], "curl": ["vort"],
           "forces": ["velX", "S", "S2"], "project": ["vel"]}


@pytest.mark.parametrize("stage", ["adv1", "adv2", "curl", "forces", "project"])
def test_stage_parity(campfire, stage):
    sim, orc, dt = _stage_case(campfire, stage, params={"windX": 0.6, "windZ": -0.3, "gust": 0.5})
    if stage == "project":
        p = (FC.smooth_noise(FC.C1["res"][::-1], np.random.default_rng(5)) * 0.02).astype(np.float32)
        sim.set_level(0, "p", p)
        orc.put_level(0, "p", p)
    sim.run_stage(stage, dt)
    sim.sync()
    if stage == "forces":
        orc.stage("curl")   # the GPU forces kernel computes the curl itself
    orc.stage(stage)
    for name in OUTPUTS[stage]:
        g, o = sim.download(name), orc.get(name)
        for c in range(4):
            FC.compare(g[..., c], o[..., c], RTOL, ATOL, OUTLIERS, what=f"{stage}:{name}[{c}]")


@pytest.mark.parametrize("case", ["burst", "visc_lam", "spots", "low_intensity"])
def test_forces_variants(campfire, case):
    params, spots = {}, None
    if case == "burst":
        params = {"burstX": 0.02, "burstY": 0.08, "burstZ": -0.03, "burstAmt": 1.0, "seed": 3.0}
    elif case == "visc_lam":
        params = {"visc": 1.0, "lamAge": 0.2}
    elif case == "spots":
        spots = F.make_spots(11, 3, 2.0, 2.0, 0.02, 0.15)
    else:
        params = {"intensity": 0.2}
    sim, orc, dt = _stage_case(campfire, "forces", params=params, spots=spots, seed=8)
    sim.run_stage("forces", dt)
    sim.sync()
    orc.stage("curl")
    orc.stage("forces")
    for name in OUTPUTS["forces"]:
        g, o = sim.download(name), orc.get(name)
        for c in range(4):
            FC.compare(g[..., c], o[..., c], RTOL, ATOL, OUTLIERS, what=f"forces/{case}:{name}[{c}]")


def test_div_parity(campfire):
    sim, orc, dt = _stage_case(campfire, "div")
    sim.run_stage("div", dt)
    sim.sync()
    orc.stage("div")
    FC.compare(sim.level(0, "b"), orc.get_level(0, "b"), RTOL, ATOL, OUTLIERS, what="div")


def _mg_pair(seed=1):
    sim, orc = FC.make_pair(FC.C1)
    rng = np.random.default_rng(seed)
    for l, L in enumerate(sim.levels):
        nx, ny, nz = L["dims"]
        p = (FC.smooth_noise((nz, ny, nx), rng, 1) * 0.01).astype(np.float32)
        b = (FC.smooth_noise((nz, ny, nx), rng, 1) * 50.0).astype(np.float32)
        for w, a in (("p", p), ("b", b)):
            sim.set_level(l, w, a)
            orc.put_level(l, w, a)
    return sim, orc


@pytest.mark.parametrize("level", [0, 1, 2])
def test_mg_smooth_restrict_prolong(level):
    sim, orc = _mg_pair(level + 1)
    for color in (0, 1):
        sim.run_mg("smooth", level, color)
        orc.mg_smooth(level, color)
    sim.sync()
    FC.compare(sim.level(level, "p"), orc.get_level(level, "p"), 1e-5, 1e-6, 0, what=f"smooth L{level}")
    sim.run_mg("restrict", level)
    orc.mg_restrict(level)
    sim.sync()
    FC.compare(sim.level(level + 1, "b"), orc.get_level(level + 1, "b"), 1e-4, 1e-5, 0, what=f"restrict L{level}")
    assert not sim.level(level + 1, "p").any()
    # prolongation of a non-zero coarse field
    pc = (FC.smooth_noise(sim.levels[level + 1]["dims"][::-1], np.random.default_rng(9), 1)).astype(np.float32)
    sim.set_level(level + 1, "p", pc)
    orc.put_level(level + 1, "p", pc)
    sim.run_mg("prolong", level)
    orc.mg_prolong(level)
    sim.sync()
    FC.compare(sim.level(level, "p"), orc.get_level(level, "p"), 1e-5, 1e-6, 0, what=f"prolong L{level}")


@pytest.mark.parametrize("level,sweeps", [(0, 2), (1, 3), (2, 1)])
def test_rb_sweeps(level, sweeps):
    """`sweeps` red-black sweeps through the V-cycle path equal colour 0 then colour 1, repeated."""
    sim, orc = _mg_pair(11 + level)
    sim.run_mg("sweeps", level, sweeps)
    for _ in range(sweeps):
        orc.mg_smooth(level, 0)
        orc.mg_smooth(level, 1)
    sim.sync()
    FC.compare(sim.level(level, "p"), orc.get_level(level, "p"), 1e-5, 1e-6, 0, what=f"sweeps L{level}")


@pytest.mark.parametrize("res", [(8, 16, 8), (16, 32, 16), (12, 400, 12), (20, 30, 20), (32, 64, 32), (48, 32, 32),
                                 (64, 128, 64)])
def test_mg_vcycle_tail_shapes(res):
    """V-cycles whose shared-memory tail has only warp-sized levels (8x16x8), only CTA-sized levels (12x400x12:
    coarsest 6x200x6), an odd coarsest level (20x30x20 -> 10x15x10), cluster tails (16x32x16: one distributed
    level over gathered levels), and launch-per-phase levels above the tail (32x64x32 up to 64x128x64;
    48x32x32 with nx not a power of two)."""
    cfg = dict(res=res, size=(0.02 * res[0], 0.02 * res[1], 0.02 * res[2]), dt=0.01, vcycles=2)
    sim, orc = FC.make_pair(cfg)
    rng = np.random.default_rng(sum(res))
    for l, L in enumerate(sim.levels):
        nx, ny, nz = L["dims"]
        for w, scale in (("p", 0.01), ("b", 50.0)):
            a = (FC.smooth_noise((nz, ny, nx), rng, 1) * scale).astype(np.float32)
            sim.set_level(l, w, a)
            orc.put_level(l, w, a)
    for _ in range(2):
        sim.run_stage("vcycle", cfg["dt"])
        orc.vcycle()
    sim.sync()
    FC.compare(sim.level(0, "p"), orc.get_level(0, "p"), 1e-4, 1e-5, 0, what=f"vcycle {res}")


@pytest.mark.parametrize("res", [(16, 32, 16), (32, 64, 32), (48, 32, 32)])
def test_mg_cluster_tail_whole_cycle(res):
    """The 8-CTA cluster tail run over the whole hierarchy (fire_sim_run_mg from level 0): one distributed level
    over gathered levels (16x32x16), two distributed levels (32x64x32; 48x32x32 with nx not a power of two)
    equal the oracle's V-cycle."""
    cfg = dict(res=res, size=(0.02 * res[0], 0.02 * res[1], 0.02 * res[2]), dt=0.01, vcycles=2)
    sim, orc = FC.make_pair(cfg)
    rng = np.random.default_rng(sum(res) + 1)
    for l, L in enumerate(sim.levels):
        nx, ny, nz = L["dims"]
        for w, scale in (("p", 0.01), ("b", 50.0)):
            a = (FC.smooth_noise((nz, ny, nx), rng, 1) * scale).astype(np.float32)
            sim.set_level(l, w, a)
            orc.put_level(l, w, a)
    for _ in range(2):
        sim.run_mg("tail", 0)
        orc.vcycle()
    sim.sync()
    FC.compare(sim.level(0, "p"), orc.get_level(0, "p"), 1e-4, 1e-5, 0, what=f"cluster tail {res}")


def test_mg_vcycle_parity():
    """One V(2,2) cycle: the shared-memory tail kernel runs the coarse levels."""
    sim, orc = _mg_pair(7)
    for _ in range(2):
        sim.run_stage("vcycle", FC.C1["dt"])
        orc.vcycle()
    sim.sync()
    FC.compare(sim.level(0, "p"), orc.get_level(0, "p"), 1e-4, 1e-5, 0, what="vcycle p0")
    r_gpu = sim.residual()
    rr, bb = orc.residual()
    assert r_gpu == pytest.approx(np.sqrt(rr / bb), rel=1e-3)
