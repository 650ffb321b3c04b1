"""The oracle's source-term stage (curl + forces, src/sim.js:200-211, 214-396) against an independent numpy
restatement of the WGSL, both in FP64, on a small grid that reaches every branch: log and coal-bed sources
with their noise lookups, a burst, ignition and burning, soot formation and oxidation, radiative and
Newtonian cooling, viscosity, the laminar base, confinement, curl noise, wind, solids, side sponge and top
fade.  This cross-checks the part of the restatement that no reference test pins."""
import numpy as np

import fire_sim as F
import numpy_fire as NF
from numpy_fire import IDX, smoothstep


def test_forces_matches_numpy_restatement(oracle_mod, tables):
    noise, curl = tables
    res, dx, dt = (12, 18, 10), 0.0125, 1.0 / 120.0
    nx, ny, nz = res
    rng = np.random.default_rng(21)
    sh = (nz, ny, nx)
    u = lambda lo, hi: rng.uniform(lo, hi, sh)
    velY = np.stack([u(-3, 3), u(-2, 4), u(-3, 3), np.zeros(sh)], -1)
    SY = np.stack([u(0, 1.6), u(0, 0.2), u(0, 3.0), u(0, 3.0)], -1)
    S2Y = np.stack([u(0, 0.9), u(0, 0.3), u(0, 0.05), u(0, 1.0)], -1)
    geo = np.zeros(sh + (4,))
    geo[:, :4, :, 0] = np.where(rng.uniform(size=(nz, 4, nx)) < 0.5, rng.uniform(0.0, 1.0, (nz, 4, nx)), 0.0)   # log surfaces
    geo[2:7, :2, 3:9, 1] = rng.uniform(0.2, 1.0, (5, 2, 6))                                                    # coal bed
    geo[4:6, 1:3, 5:7, 2] = 1.0                                                                                 # solid wood
    P = F.param_defaults().copy()
    for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("dx", dx), ("dt", dt), ("time", 1.7), ("seed", 3.0),
                 ("ox", -nx * dx / 2), ("oy", 0.0), ("oz", -nz * dx / 2), ("windX", 0.5), ("windZ", -0.3),
                 ("gust", 0.4), ("burstAmt", 0.8), ("burstX", 0.01), ("burstY", 0.05), ("burstZ", -0.01),
                 ("visc", 1.0), ("lamAge", 0.05), ("ignT", 700.0)):
        P[IDX[k]] = v
    E = np.zeros(144, np.float32)
    E[0], E[1] = 0.015, 0.05         # the reference's soot age gate smoothstep(0.015, 0.05, ageF)
    E[5] = -1e30                     # no spots
    orc = oracle_mod.OracleSim(res, float(np.float32(dx)), dbl=True)
    orc.set_params(P)
    orc.set_ext(E)
    orc.set_tables(noise, curl)
    for k, a in (("velY", velY), ("SY", SY), ("S2Y", S2Y), ("geo", geo)):
        orc.put(k, a)
    orc.stage("curl")
    orc.stage("forces")
    want_v, want_s, want_s2 = NF.forces(P, E, velY, SY, S2Y, geo, noise.astype(np.float64), curl.astype(np.float64))
    # the case reaches the branches it is meant to
    T = 293.0 + 1000.0 * SY[..., 0]
    assert (T > 1100).any() and (T < 450).any() and (geo[..., 0] > 0.001).sum() > 50
    for name, want in (("velX", want_v), ("S", want_s), ("S2", want_s2)):
        got = orc.get(name, np.float64)
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-10, err_msg=name)


def test_geo_matches_numpy_restatement(oracle_mod):
    """Emitter geometry (src/sim.js:498-523, sdCapsule src/shaders/lib.js:57-62) for the packed campfire
    (8 logs + 8 zero slots, as packLogs leaves them), against a numpy restatement in FP64.  The zero slots are
    degenerate capsules (dot(ba, ba) = 0); clamp ignores the NaN, so h = 0 there."""
    res, dx = (24, 20, 22), 0.02
    nx, ny, nz = res
    logs = oracle_mod.build_campfire(7).astype(np.float64).reshape(16, 8)
    P = F.param_defaults().copy()
    for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("dx", dx), ("ox", -nx * dx / 2), ("oy", 0.0),
                 ("oz", -nz * dx / 2), ("nLogs", 16.0)):
        P[IDX[k]] = v
    E = np.zeros(144, np.float32)
    E[2] = 1.0                       # coal-bed gain 1: the reference's bed
    E[5] = -1e30
    orc = oracle_mod.OracleSim(res, float(np.float32(dx)), dbl=True)
    orc.set_params(P)
    orc.set_ext(E)
    orc.set_logs(logs.astype(np.float32).ravel())
    orc.stage("geo")
    got = orc.get("geo", np.float64)

    g = lambda n: float(P[IDX[n]])
    dxd = g("dx")
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    p = np.array([g("ox"), g("oy"), g("oz")]) + (np.stack([i, j, k], -1) + 0.5) * dxd
    rxz = np.linalg.norm(p[..., [0, 2]], axis=-1)
    lg = logs.astype(np.float32).astype(np.float64)
    dmin = np.full(p.shape[:-1], 1e9)
    band = np.zeros(p.shape[:-1])
    for n in range(int(g("nLogs"))):
        a, r, bb, burn = lg[n, 0:3], lg[n, 3], lg[n, 4:7], lg[n, 7]
        pa, ba = p - a, bb - a
        with np.errstate(invalid="ignore", divide="ignore"):
            h = np.fmin(np.fmax((pa @ ba) / (ba @ ba), 0.0), 1.0)      # NaN-ignoring clamp
        dd = np.linalg.norm(pa - h[..., None] * ba, axis=-1) - r
        dd = dd + r * 0.3 * (1.0 - smoothstep(0.0, 0.16, rxz)) * burn
        dmin = np.minimum(dmin, dd)
        bnd = 1.0 - smoothstep(0.0, 1.6 * dxd, np.abs(dd - 0.6 * dxd))
        hot = burn * (1.0 - smoothstep(g("hotR0"), g("hotR1"), rxz)) * (1.0 - smoothstep(0.08, g("hotY1"), p[..., 1]))
        band = np.maximum(band, bnd * hot)
    bedH = 0.05 * (1.0 - smoothstep(0.0, g("bedRadius"), rxz)) + 0.02
    bed = ((1.0 - smoothstep(0.0, 2.0 * dxd, p[..., 1] - bedH)) *
           (1.0 - smoothstep(g("bedRadius") * 0.6, g("bedRadius") * 1.15, rxz)))
    solid = np.where(dmin < -0.5 * dxd, 1.0, 0.0)
    want = np.stack([band, bed, solid, dmin], -1)
    assert band.max() > 0.5 and bed.max() > 0.5 and solid.sum() > 10
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12)


def test_whole_step_matches_numpy_restatement(oracle_mod, tables):
    """One full step (src/sim.js:627-648: adv1, adv2, curl + forces, div, two V(2,2) cycles from the previous
    pressure, project) of the oracle's FP64 mode against the numpy stages composed in the reference's order."""
    noise, curl = tables
    res, dx = (16, 24, 16), 0.0125
    nx, ny, nz = res
    rng = np.random.default_rng(51)
    sh = (nz, ny, nx)
    u = lambda lo, hi: rng.uniform(lo, hi, sh)
    state = {"vel": np.stack([u(-2, 2), u(-1, 3), u(-2, 2), np.zeros(sh)], -1),
             "S": np.stack([u(0, 1.5), u(0, 0.2), u(0, 2.0), u(0, 2.0)], -1),
             "S2": np.stack([u(0, 0.9), u(0, 0.3), u(0, 0.05), u(0, 1.0)], -1),
             "p": rng.normal(0, 0.01, sh)}
    geo = np.zeros(sh + (4,))
    geo[:, :5, :, 0] = np.where(rng.uniform(size=(nz, 5, nx)) < 0.4, rng.uniform(0, 1, (nz, 5, nx)), 0.0)
    geo[5:11, :2, 5:11, 1] = 0.8
    geo[7:9, 1:3, 7:9, 2] = 1.0
    P = F.param_defaults().copy()
    for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("dx", dx), ("dt", 1.0 / 120.0), ("time", 0.9), ("seed", 2.0),
                 ("ox", -nx * dx / 2), ("oy", 0.0), ("oz", -nz * dx / 2), ("windX", 0.3), ("ignT", 700.0)):
        P[IDX[k]] = v
    E = np.zeros(144, np.float32)
    E[0], E[1], E[5] = 0.015, 0.05, -1e30
    orc = oracle_mod.OracleSim(res, float(np.float32(dx)), dbl=True)
    orc.set_params(P)
    orc.set_ext(E)
    orc.set_tables(noise, curl)
    for k in ("vel", "S", "S2"):
        orc.put(k, state[k])
    orc.put("geo", geo)
    orc.put_level(0, "p", state["p"])
    orc.step_raw(False, 2)
    want = NF.step(P, E, state, geo, noise.astype(np.float64), curl.astype(np.float64), orc.levels, orc.coarse_iters, 2)
    for k in ("vel", "S", "S2", "velX"):
        got = orc.get(k, np.float64)
        scale = np.abs(want[k]).max()
        np.testing.assert_allclose(got, want[k], rtol=1e-8, atol=1e-10 * scale, err_msg=k)
    np.testing.assert_allclose(orc.get_level(0, "p", np.float64), want["p"], rtol=1e-8, atol=1e-10 * np.abs(want["p"]).max())
