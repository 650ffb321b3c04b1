"""Shared helpers for the parity tests: the configured workloads and identical GPU / oracle set-ups."""
from __future__ import annotations

import numpy as np

import fire_sim as F
import oracle as O

# Reference-emitter parity grid: 48x96x48 at 1.25 cm (0.6 x 1.2 x 0.6 m), dt = 1/120, 4 V-cycles.
C1 = dict(res=(48, 96, 48), size=(0.6, 1.2, 0.6), dt=1.0 / 120.0, vcycles=4)
# Full-physics throughput grid: 128x256x128 at 5 mm, dt = 1/240.
C2 = dict(res=(128, 256, 128), size=(0.64, 1.28, 0.64), dt=1.0 / 240.0, vcycles=4)

FIELD_NAMES = ["vel", "velX", "velY", "S", "SX", "SY", "S2", "S2X", "S2Y", "vort", "geo"]


def smooth_noise(shape, rng, passes=3):
    """Band-limited random field in [-1, 1] (box-filtered white noise), shape (z, y, x)."""
    a = rng.standard_normal(shape).astype(np.float64)
    for _ in range(passes):
        for ax in range(3):
            a = (np.roll(a, 1, ax) + a + np.roll(a, -1, ax)) / 3.0
    a /= max(np.abs(a).max(), 1e-12)
    return a


def random_state(res, seed=0):
    """A plausible mid-burn state: smooth velocities of a few m/s and scalars in their physical ranges."""
    nx, ny, nz = res
    rng = np.random.default_rng(seed)
    sh = (nz, ny, nx)
    n = lambda: smooth_noise(sh, rng)
    pos = lambda s: np.clip(0.5 + 0.5 * n(), 0, 1) * s
    vel = np.stack([2.0 * n(), 1.0 + 2.5 * n(), 2.0 * n(), np.zeros(sh)], -1)
    S = np.stack([pos(1.4), pos(0.15), pos(4.0), pos(3.0)], -1)
    S2 = np.stack([pos(0.9), pos(0.2), pos(0.05), pos(1.0)], -1)
    hats = [np.clip(a + 0.05 * np.stack([n() for _ in range(4)], -1), 0 if i else -1e9, 1e9)
            for i, a in enumerate((vel, S, S2))]
    hats[0][..., 3] = 0.0
    velY = np.stack([2.0 * n(), 1.0 + 2.5 * n(), 2.0 * n(), np.zeros(sh)], -1)
    SY = np.stack([pos(1.4), pos(0.15), pos(4.0), pos(3.0)], -1)
    S2Y = np.stack([pos(0.9), pos(0.2), pos(0.05), pos(1.0)], -1)
    st = dict(vel=vel, velX=hats[0], S=S, SX=hats[1], S2=S2, S2X=hats[2], velY=velY, SY=SY, S2Y=S2Y)
    return {k: np.ascontiguousarray(v, np.float32) for k, v in st.items()}


def make_pair(cfg, logs=None, dbl=False, spots=None, soot_age=None, bed_gain=None, params=None):
    """A GPU FireSim and an oracle configured identically (tables copied from the GPU)."""
    sim = F.FireSim(res=cfg["res"], size=cfg["size"], logs=logs, vcycles=cfg["vcycles"])
    if params:
        sim.set_params(params)
    if spots is not None:
        sim.set_spots(spots)
    if soot_age is not None:
        sim.set_soot_age(*soot_age)
    if bed_gain is not None:
        sim.set_bed_gain(bed_gain)
    orc = O.OracleSim(cfg["res"], sim.dx, dbl=dbl)
    orc.set_tables(sim.download("noise").astype(np.float32), sim.download("curl").astype(np.float32))
    orc.set_logs(logs if logs is not None else np.zeros(0, np.float32))
    return sim, orc


def sync_block(sim, orc, dt):
    """Gives the oracle exactly the block the GPU uses for its next stage/step."""
    blk = sim.peek_block(dt)
    orc.set_params(blk[:64])
    orc.set_ext(blk[64:])
    return blk


def put_state(sim, orc, state):
    for k, v in state.items():
        sim.upload(k, v)
        orc.put(k, v)


def compare(a, b, rtol, atol_frac, max_outlier_frac=0.0, what=""):
    """|a - b| <= atol + rtol |b| with atol = atol_frac * max|b|, allowing a small fraction of outliers."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert np.isfinite(a).all(), f"{what}: non-finite GPU values"
    scale = max(np.abs(b).max(), 1e-30)
    tol = atol_frac * scale + rtol * np.abs(b)
    err = np.abs(a - b)
    bad = err > tol
    frac = bad.mean()
    assert frac <= max_outlier_frac, (
        f"{what}: {bad.sum()} / {bad.size} cells beyond tolerance (max err {err.max():.3e}, scale {scale:.3e})")
    return float(err.max() / scale)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
