"""The cinematic's timeline (src/timeline.js) against an independent Python restatement with JavaScript
number semantics, and the capture-mode driver (capStep, src/main.js:153-160) on a live simulation."""
import math

import numpy as np
import pytest

import fire_cases as FC

SCRIPTED = [  # (t, type, strength, pos, aim)   src/timeline.js:34-47
    (0.30, "pop", 1.0, (0.06, 0.14, 0.12), (0.5, 0, 0.86)), (2.433, "pop", 0.5, (-0.08, 0.12, 0.10), None),
    (4.6, "pop", 0.6, (0.10, 0.16, 0.02), None), (5.633, "pop", 0.45, (-0.05, 0.10, 0.12), None),
    (7.2, "crackle-burst", 0.5, (-0.10, 0.08, 0.06), None), (8.433, "pop", 0.5, (0.06, 0.12, 0.10), None),
    (9.0, "log-shift", 1.0, (0.05, 0.12, 0.0), None), (11.0, "gust", 1.0, (0, 0.3, 0), None),
    (13.433, "pop", 0.5, (0.08, 0.13, -0.05), None), (15.2, "pop", 0.85, (-0.06, 0.15, 0.08), None),
    (16.633, "pop", 0.5, (0.02, 0.12, 0.12), None), (18.5, "pop", 1.0, (0.06, 0.14, 0.12), (0.5, 0, 0.86)),
]


def _to_fixed(x, d):
    return float(f"{x:.{d}f}")


def _random_pops(seed=20261025):
    st = seed & 0xFFFFFFFF
    def rnd():
        nonlocal st
        st = (st * 1664525 + 1013904223) & 0xFFFFFFFF
        return st / 4294967296
    out, t = [], 0.6
    while t < 20 - 0.3:
        t += -math.log(1 - rnd()) / 0.8
        if t >= 20 - 0.3:
            break
        strength = min(0.6, 0.12 + 0.45 * rnd() ** 2.2)
        a, r = rnd() * math.pi * 2, math.sqrt(rnd()) * 0.2
        out.append((_to_fixed(t, 3), "pop", _to_fixed(strength, 2), (math.cos(a) * r, 0.07 + rnd() * 0.15, math.sin(a) * r), None))
        if rnd() < 0.25:
            t2 = t + 0.05 + rnd() * 0.25
            out.append((_to_fixed(t2, 3), "pop", _to_fixed(strength * 0.5, 2), (math.cos(a) * r, 0.1, math.sin(a) * r), None))
    return [e for e in out if not any(abs(s[0] - e[0]) < 0.35 for s in SCRIPTED)]


EVENTS = sorted(SCRIPTED + _random_pops(), key=lambda e: e[0])   # Python's sort is stable, as V8's
INTENSITY = [(-5.0, 1.0), (0.0, 1.0), (1.0, 1.0), (2.0, 1.12), (6.0, 1.12), (8.6, 1.0), (9.0, 1.2), (9.6, 1.05),
             (11.0, 1.08), (12.6, 1.08), (14.0, 1.05), (18.3, 1.05), (18.5, 1.15), (19.2, 1.0), (20.0, 1.0)]


def _intensity(t):
    k = INTENSITY
    if t <= k[0][0]:
        return k[0][1]
    for i in range(len(k) - 1):
        if t <= k[i + 1][0]:
            u = (t - k[i][0]) / (k[i + 1][0] - k[i][0])
            return k[i][1] + (k[i + 1][1] - k[i][1]) * u * u * (3 - 2 * u)
    return k[-1][1]


def _sim_at(t):
    p = {"intensity": _intensity(t), "burstAmt": 0.0, "burstX": 0.0, "burstY": 0.0, "burstZ": 0.0}
    for (et, ty, s, pos, _) in EVENTS:
        dt = t - et
        if dt < 0 or dt > 0.4:
            continue
        if ty in ("log-shift", "pop", "crackle-burst"):
            w = (1.0 if ty == "log-shift" else 0.6) * s * math.exp(-dt / (0.12 if ty == "log-shift" else 0.04))
            if w > p["burstAmt"]:
                p["burstAmt"], (p["burstX"], p["burstY"], p["burstZ"]) = w, pos
    p["windX"] = 0.28 * math.sin(t * 0.23 + 1.0) + 0.14 * math.sin(t * 0.61 + 0.4)
    p["windZ"] = 0.18 * math.sin(t * 0.17 + 2.3)
    dt = t - 11.0
    w = math.sin(math.pi * min(dt / 2.2, 1)) ** 1.5 if 0 < dt < 2.8 else 0.0
    p["windX"] += 2.8 * w
    return p


def test_events_match_restatement():
    import fire_sim as F
    got = F.timeline_events()
    assert len(got) == len(EVENTS)
    for g, (t, ty, s, pos, aim) in zip(got, EVENTS):
        assert g["t"] == t and g["type"] == ty and g["strength"] == s, (g, t, ty, s)
        np.testing.assert_allclose(g["pos"], pos, rtol=0, atol=1e-12)
        assert (g["aim"] is None) == (aim is None)


@pytest.mark.parametrize("t", [-3.0, 0.0, 0.31, 1.4, 2.2, 7.25, 9.0, 9.05, 9.3, 11.5, 12.9, 18.6, 19.95, 25.0])
def test_sim_at_matches_restatement(t):
    import fire_sim as F
    got, want = F.timeline_sim_at(t), _sim_at(t)
    for k, v in want.items():
        assert got[k] == pytest.approx(v, rel=1e-12, abs=1e-12), (t, k)
    assert F.timeline_intensity_at(t) == pytest.approx(_intensity(t), rel=1e-12)


def test_log_offsets_and_lens():
    import fire_sim as F
    assert F.timeline_log_offsets_at(8.99) is None
    o = F.timeline_log_offsets_at(9.06)
    u = 0.06 / 0.12
    assert o["index"] == 3 and o["s"] == pytest.approx(u * u * (3 - 2 * u)) and o["topDrop"] == 0.04
    assert F.timeline_log_offsets_at(12.0)["s"] == 1.0
    c = F.timeline_camera_at(0.0)
    assert c["fov"] == 42.0 and np.linalg.norm(np.subtract(c["pos"], (0.62, 0.30, 1.05))) < 0.01
    L = F.timeline_lens_at(0.0)
    fmm = 18 / math.tan(math.radians(42) / 2)
    assert L["fmm"] == pytest.approx(fmm) and L["aperture"] == pytest.approx(fmm / 16.0 / 1000.0) and L["N"] == 8.0


# ------------------------------------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def campfire():
    import fire_sim as F
    return F.build_campfire(7)


@pytest.mark.gpu
def test_driver_applies_cue_sheet(campfire):
    """Steps through the log shift at 9.0 s: every step's parameter block carries simAt(t), the moved log
    rebuilds the emitter geometry, and the event's spark burst is thrown."""
    import fire_sim as F
    sim = F.FireSim(res=FC.C1["res"], size=FC.C1["size"], logs=campfire, vcycles=4)
    sparks = F.Sparks(sim, count=2048)
    tl = F.Timeline(campfire, steps_per_frame=4)
    j0 = int(round(8.9 * 30 * 4))
    geo0 = None
    for j in range(j0, j0 + 40):
        t = tl.time(j)
        tl.step(sim, j, sparks)
        blk = sim.peek_block(tl.dt)
        want = F.timeline_sim_at(t)
        for name in ("intensity", "burstAmt", "windX", "windZ"):
            assert blk[F.SIM_FIELDS.index(name)] == pytest.approx(np.float32(want[name]), rel=1e-6, abs=1e-7), (t, name)
        if j == j0:
            sim.sync()
            geo0 = sim.download("geo").copy()
    sim.sync()
    assert not np.array_equal(sim.download("geo"), geo0)         # the shifted log moved the emitter
    assert (sparks.download()[:, 14] > 0.5).sum() > 50           # the log-shift burst is in the air
    tl.close()
    sparks.close()
    sim.close()
