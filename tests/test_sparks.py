"""Sparks (src/sparks.js): the CPU restatement's spawn pinned by an independent Python restatement, and the
CUDA particle update against the restatement step by step, from identical state, on a burning fire."""
import math

import numpy as np
import pytest

import fire_cases as FC

M32 = 0xFFFFFFFF


def _pcg1(n):
    s = (n * 747796405 + 2891336453) & M32
    w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & M32
    return (w >> 22) ^ w


def _rand2(n, m):   # lib.js:18, f32(u32) * f32(1 / 4294967295)
    return np.float32(np.float32(_pcg1((n ^ _pcg1(m)) & M32)) * np.float32(2.0 ** -32))


def _spawn_py(slot, U):
    """The non-burst spawn of sparks.js:98-111 in Python (float64 arithmetic on the f32 random numbers)."""
    seed, frame = int(U[20]), int(U[2])
    r = lambda k: float(_rand2((slot * 7919 + k * 104729 + seed) & M32, frame))
    gauss = lambda k: math.sqrt(-2.0 * math.log(max(r(k), 1e-6))) * math.cos(6.2831853 * r(k + 1))
    a, rr = r(1) * 6.2831853, math.sqrt(r(2)) * U[19]
    p = (math.cos(a) * rr, 0.05 + r(3) * 0.12, math.sin(a) * rr)
    v = (gauss(4) * 0.4, 0.6 + r(6) * 1.8, gauss(11) * 0.4)
    dmm = min(max(0.5 * math.exp(0.55 * gauss(13)) * U[21], 0.15), 2.5)
    tb = (0.25 + 2.0 * dmm * dmm) * (0.6 + 0.8 * r(15)) * U[18]
    T0 = 1230.0 + 70.0 * gauss(16)
    fl = 5.0 + 15.0 * r(18) if r(20) < 0.45 else 0.0
    return [*p, 0.0, *v, tb, *p, T0, dmm, r(19), 1.0, fl]


def _uniforms(nBase=0, nBurst=0, frame=3, dt=1 / 120, time=0.5):
    U = np.zeros(27, np.float32)
    U[0], U[1], U[2], U[3], U[4], U[5] = dt, time, frame, 16, nBase, nBurst
    U[11:17] = (-0.3, 0.0, -0.3, 0.6, 1.2, 0.6)     # box origin and size
    U[17], U[18], U[19], U[20], U[21], U[22], U[24] = 1.0, 1.0, 0.2, 1234.0, 1.0, 1.0, 1.0
    return U


def test_oracle_spawn_matches_python(oracle_mod):
    """Base spawns of the restatement equal an independent Python restatement; slots go to dead sparks in
    index order and stop at nBase + nBurst."""
    sp = np.zeros((16, 16), np.float32)
    sp[[2, 5], 14] = 1.0                  # two live sparks are skipped by the slot count
    sp[[2, 5], 1] = 0.5
    sp[[2, 5], 11] = 1000.0
    sp[[2, 5], 7] = 1.0
    sp[[2, 5], 12] = 0.5
    U = _uniforms(nBase=5)
    vel = np.zeros((4, 8, 4, 4), np.float32)
    curl = np.zeros((4, 4, 4, 4), np.float32)
    out = oracle_mod.sparks_step(sp, U, vel, curl)
    dead = [i for i in range(16) if i not in (2, 5)]
    for slot, i in enumerate(dead):
        if slot < 5:
            np.testing.assert_allclose(out[i], _spawn_py(slot, U), rtol=2e-5, atol=2e-6)
        else:
            assert out[i, 14] == 0.0 and not out[i].any()
    assert (out[[2, 5], 14] == 1.0).all()


# ------------------------------------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def campfire():
    import fire_sim as F
    return F.build_campfire(7)


@pytest.mark.gpu
def test_sparks_match_oracle(oracle_mod, campfire):
    import fire_sim as F
    dt = FC.C1["dt"]
    sim = F.FireSim(res=FC.C1["res"], size=FC.C1["size"], logs=campfire, vcycles=4)
    sim.step(dt, 40)
    sp = F.Sparks(sim, count=2048)
    sp.set(rate=60.0)
    sp.burst(n=120, pos=(0.05, 0.12, 0.0), speed=4.5, radius=0.12, dur=0.15, fan=0.7, size=1.5)
    sp.burst(n=80, pos=(0.06, 0.14, 0.12), speed=5.0, radius=0.03, dur=0.05, fan=0.9, size=1.4, aim=(0.5, 0.0, 0.86))
    curl = sim.download("curl").astype(np.float32)
    worst, flips, alive = 0.0, 0, 0
    for k in range(24):
        sim.step(dt, 1)
        sim.sync()
        before = sp.download()
        U = sp.peek(dt)
        vel = sim.download("vel")
        sp.step(dt)
        got = sp.download()
        want = oracle_mod.sparks_step(before, U, vel, curl)
        both = (got[:, 14] == want[:, 14])
        flips += int((~both).sum())
        live = both & (want[:, 14] > 0.5)
        if live.any():
            scale = np.maximum(np.abs(want[live]), 1.0)
            worst = max(worst, float((np.abs(got[live] - want[live]) / scale).max()))
        alive = int((got[:, 14] > 0.5).sum())
    assert alive > 100, alive                  # bursts and the base rate are in the air
    assert flips <= 2, flips                   # a kill threshold can flip on an ulp of exp/log/cos
    assert worst < 1e-4, worst
    sp.close()
    sim.close()


@pytest.mark.gpu
def test_sparks_deterministic(campfire):
    import fire_sim as F
    dt = FC.C1["dt"]
    runs = []
    for _ in range(2):
        sim = F.FireSim(res=FC.C1["res"], size=FC.C1["size"], logs=campfire, vcycles=4)
        sp = F.Sparks(sim, count=1024)
        sp.set(rate=80.0)
        sp.burst(n=60, pos=(0.0, 0.12, 0.0), speed=3.0, radius=0.05, dur=0.1)
        for _ in range(12):
            sim.step(dt, 1)
            sp.step(dt)
        runs.append(sp.download())
        sp.reset()
        assert not sp.download().any()
        sp.close()
        sim.close()
    assert np.array_equal(runs[0], runs[1])
