"""The oracle's source-term stage (curl + forces, src/sim.js:200-211, 214-396) against an independent numpy
restatement of the WGSL, both in FP64, on a small grid that reaches every branch: log and coal-bed sources
with their noise lookups, a burst, ignition and burning, soot formation and oxidation, radiative and
Newtonian cooling, viscosity, the laminar base, confinement, curl noise, wind, solids, side sponge and top
fade.  This cross-checks the part of the restatement that no reference test pins."""
import numpy as np
import pytest

import fire_sim as F

IDX = {n: i for i, n in enumerate(F.SIM_FIELDS)}


def smoothstep(e0, e1, x):
    t = np.clip((x - e0) / (e1 - e0), 0.0, 1.0)
    return t * t * (3.0 - 2.0 * t)


def mix(a, b, t):
    return a * (1.0 - t) + b * t


def sample_repeat(tab, q):
    """textureSampleLevel with a linear, repeat sampler on an N^3 table at normalised coordinates q."""
    N = tab.shape[0]
    u = q * N - 0.5
    fl = np.floor(u)
    f = u - fl
    i0 = fl.astype(np.int64) % N
    out = np.zeros(q.shape[:-1] + (4,))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = ((f[..., 0] if dx else 1 - f[..., 0]) * (f[..., 1] if dy else 1 - f[..., 1]) *
                     (f[..., 2] if dz else 1 - f[..., 2]))
                out += w[..., None] * tab[(i0[..., 2] + dz) % N, (i0[..., 1] + dy) % N, (i0[..., 0] + dx) % N]
    return out


def ld(f, di, dj, dk):
    """textureLoad at the clamped neighbour (i + di, j + dj, k + dk) of every cell."""
    nz, ny, nx = f.shape[:3]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return f[np.clip(k + dk, 0, nz - 1), np.clip(j + dj, 0, ny - 1), np.clip(i + di, 0, nx - 1)]


def curl_field(vel):
    L, R = ld(vel, -1, 0, 0), ld(vel, 1, 0, 0)
    B, T = ld(vel, 0, -1, 0), ld(vel, 0, 1, 0)
    K, Fw = ld(vel, 0, 0, -1), ld(vel, 0, 0, 1)
    w = np.stack([(T[..., 2] - B[..., 2]) - (Fw[..., 1] - K[..., 1]),
                  (Fw[..., 0] - K[..., 0]) - (R[..., 2] - L[..., 2]),
                  (R[..., 1] - L[..., 1]) - (T[..., 0] - B[..., 0])], -1) * 0.5
    return np.concatenate([w, np.linalg.norm(w, axis=-1)[..., None]], -1)


def forces_numpy(P, E, velY, SY, S2Y, geo, noise, curl):
    g = lambda n: float(P[IDX[n]])
    nz, ny, nx = SY.shape[:3]
    dt, dx, I, seed, time = g("dt"), g("dx"), g("intensity"), g("seed"), g("time")
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    fp = np.stack([i, j, k], -1) + 0.5
    p = np.array([g("ox"), g("oy"), g("oz")]) + fp * dx
    v = velY[..., :3].copy()
    s = SY.copy()
    s2 = S2Y.copy()
    noise4 = lambda q: sample_repeat(noise, q) * 2.0 - 1.0

    # sources
    qa = p * g("anchorFreq") + np.array([seed * 0.37, 0.0, 0.11])
    anchor_all = smoothstep(-0.05, 0.25, noise4(qa)[..., 2])
    qn = p * (g("srcFreq") * 0.06) + np.array([seed * 0.131, 0.0, time * g("srcSpeed")])
    th = g("srcThresh")
    pulse = smoothstep(th - 0.25, th + 0.25, noise4(qn)[..., 0])
    src_all = np.clip(geo[..., 0] * g("logSrc") * (g("srcFloor") + g("anchorGain") * anchor_all) *
                      mix(0.55, 1.0, pulse) * 1.2, 0.0, 1.0) * I
    src_all = src_all * (1.0 - geo[..., 2])
    has = geo[..., 0] > 0.001
    src = np.where(has, src_all, 0.0)
    anchor = np.where(has, anchor_all, 0.0)
    srcW = np.minimum(src, 1.0)
    bedHot = geo[..., 1]
    bed = geo[..., 1] * min(max(I * 1.4, 0.3), 1.0)
    qb = p * 2.4 + np.array([0.17, -time * 0.12, time * 0.05])
    bed = np.where(bed > 0.001, bed * smoothstep(0.0, 0.3, noise4(qb)[..., 1]), bed)
    s[..., 1] = np.maximum(s[..., 1], src * g("fuelSrc"))
    s[..., 1] = np.maximum(s[..., 1], bed * g("bedFuel"))
    s[..., 0] = np.maximum(s[..., 0], src * g("srcTemp"))
    s[..., 0] = np.maximum(s[..., 0], bedHot * g("bedTemp"))
    srcAll = np.maximum(srcW, bed)
    s2[..., 3] = mix(s2[..., 3], 1.0, bed * (1.0 - srcW))
    s2[..., 3] = mix(s2[..., 3], 0.0, srcW)
    s2[..., 1] = s2[..., 1] * (1.0 - srcAll)
    s2[..., 0] = np.maximum(s2[..., 0], (1.0 - s[..., 1]) * srcW)
    s2[..., 0] = np.maximum(s2[..., 0], (1.0 - s[..., 1]) * bed * 0.6)
    wsrc = 1.0 - np.power(1.0 - np.clip(srcW + bed * 0.4, 0.0, 1.0) * 0.5, dt * 90.0)
    v[..., 1] = mix(v[..., 1], np.maximum(v[..., 1], g("srcVel")), wsrc)
    s2[..., 2] += geo[..., 0] * (1.0 - anchor) * g("smolder") * dt * I

    # burst
    if g("burstAmt") > 0.0:
        bd = np.linalg.norm(p - np.array([g("burstX"), g("burstY"), g("burstZ")]), axis=-1)
        bw = np.clip(np.exp(-bd * bd / 0.006) * g("burstAmt"), 0.0, 1.0)
        s[..., 1] = np.maximum(s[..., 1], 0.17 * bw)
        s[..., 0] = np.maximum(s[..., 0], 0.9 * bw)
        s2[..., 0] *= 1.0 - bw
        s2[..., 3] *= 1.0 - bw
        s2[..., 1] = np.maximum(s2[..., 1], 0.05 * bw * np.clip(s[..., 1] + s2[..., 0], 0.0, 1.0))
    ageF = s2[..., 1] / np.maximum(s[..., 1] + s2[..., 0], 1e-4)

    # combustion
    T0 = 293.0 + 1000.0 * s[..., 0]
    o = np.clip(1.0 - s[..., 1] - s2[..., 0], 0.0, 1.0)
    ign = smoothstep(g("ignT") - 50.0, g("ignT") + 50.0, T0)
    b = np.minimum(s[..., 1], o / g("rs")) * (1.0 - np.exp(-g("kMix") * ign * dt))
    s[..., 1] -= b
    s2[..., 0] = np.minimum(s2[..., 0] + (1.0 + g("rs")) * b, 1.0)
    dT = np.minimum(g("heatOut") * b, np.maximum(2100.0 - T0, 0.0))
    T = T0 + dT
    q = dT / dt
    phi = np.where(geo[..., 2] > 0.5, 0.0, np.minimum(g("expansion") * q / T, 60.0))

    # soot
    ageF = np.minimum(ageF + dt, 4.0)
    s[..., 2] += (g("sootForm") * b * smoothstep(float(E[0]), float(E[1]), ageF) * smoothstep(1000.0, 1400.0, T) *
                  (1.0 - s2[..., 3]))
    s[..., 2] *= np.exp(-g("sootOx") * (0.25 + o) * smoothstep(1100.0, 1400.0, T) * dt)
    s[..., 2] *= np.exp(-g("sootOx") * 0.5 * o * smoothstep(850.0, 1100.0, T) * (1.0 - smoothstep(1100.0, 1300.0, T)) * dt)
    s[..., 2] *= np.exp(-g("sootDissip") * dt)

    # cooling
    tk = T * 0.001
    T = T - np.minimum(g("radCool") * 970.0 * s[..., 2] * tk * tk * (tk ** 4 - 0.00737), 6000.0) * dt
    notBurning = 1.0 - smoothstep(500.0, 5000.0, q)
    T = 293.0 + np.maximum(T - 293.0, 0.0) * np.exp(-g("coolRate") * notBurning * dt)
    s[..., 0] = (T - 293.0) * 0.001
    s[..., 3] = q * 1e-4
    s[..., 1] *= np.exp(-g("fuelDissip") * dt)
    s2[..., 0] *= np.exp(-g("vitDecay") * dt)
    s2[..., 2] *= np.exp(-g("smokeDissip") * dt)
    s2[..., 1] = ageF * np.clip(s[..., 1] + s2[..., 0], 0.0, 1.0)

    # buoyancy, viscosity, laminar base
    v[..., 1] += g("buoyancy") * s[..., 0] * dt
    if g("visc") > 0.0:
        lap = sum(ld(velY, *d)[..., :3] for d in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)))
        lap = lap - 6.0 * velY[..., :3]
        nu = g("visc") * 1.5e-5 * np.power(np.maximum(T, 293.0) / 293.0, 1.7)
        v += np.minimum(nu * dt / (dx * dx), 0.15)[..., None] * lap
    lam = smoothstep(0.5 * g("lamAge"), max(g("lamAge"), 1e-3), ageF) if g("lamAge") > 0.0 else np.ones_like(ageF)

    # confinement
    vort = curl_field(velY)
    grad = np.stack([ld(vort, 1, 0, 0)[..., 3] - ld(vort, -1, 0, 0)[..., 3],
                     ld(vort, 0, 1, 0)[..., 3] - ld(vort, 0, -1, 0)[..., 3],
                     ld(vort, 0, 0, 1)[..., 3] - ld(vort, 0, 0, -1)[..., 3]], -1)
    gl = np.linalg.norm(grad, axis=-1)
    gate = smoothstep(450.0, 900.0, T) * (1.0 - srcAll) * smoothstep(0.02, 0.08, p[..., 1]) * lam
    n = grad / np.where(gl > 0, gl, 1.0)[..., None]
    v += np.where((gl > 1e-6)[..., None], g("vortEps") * gate[..., None] * np.cross(n, vort[..., :3]) * dt, 0.0)

    # curl noise
    tq = (p - np.array([0.0, time * g("turbRise"), 0.0])) * g("turbFreq") + np.array([0.0, 0.0, time * g("turbEvolve")])
    cn = sample_repeat(curl, tq)[..., :3]
    tgate = (np.maximum(smoothstep(500.0, 1100.0, T), smoothstep(0.0, 3.0, s[..., 3])) * (1.0 - srcAll) *
             mix(0.6, 1.8, smoothstep(0.2, 0.75, p[..., 1])) * lam)
    v += cn * (g("turbAmp") / 12.0) * tgate[..., None] * dt * 10.0

    # wind
    windK = smoothstep(0.05, 0.5, p[..., 1]) * (1.0 + g("gust"))
    v[..., 0] += (g("windX") * windK - v[..., 0]) * dt * 0.35 * windK
    v[..., 2] += (g("windZ") * windK - v[..., 2]) * dt * 0.35 * windK
    v *= np.exp(-g("velDissip") * dt)

    # solids, sponge, top fade, speed cap
    solid = geo[..., 2] > 0.5
    v[solid] = 0.0
    s[solid, 1] = 0.0
    s2[solid, 1] = 0.0
    side = np.minimum(np.minimum(fp[..., 0], nx - fp[..., 0]), np.minimum(fp[..., 2], nz - fp[..., 2]))
    sp = (1.0 - smoothstep(0.0, 5.0, side)) * g("sponge")
    ws = smoothstep(0.03, 0.4, p[..., 1])
    ks = 1.0 - np.power(1.0 - 0.15 * np.clip(sp, 0.0, 1.0), dt * 90.0)
    v[..., 0] = mix(v[..., 0], g("windX") * ws, ks)
    v[..., 2] = mix(v[..., 2], g("windZ") * ws, ks)
    top = smoothstep(ny - 10.0, float(ny), fp[..., 1])
    kt = np.power(1.0 - 0.1 * top, dt * 90.0)
    s[..., 2] *= kt
    s2[..., 2] *= kt
    vl = np.linalg.norm(v, axis=-1)
    v = np.where((vl > 15.0)[..., None], v * (15.0 / np.where(vl > 0, vl, 1.0))[..., None], v)
    return np.concatenate([v, phi[..., None]], -1), s, s2


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
    want_v, want_s, want_s2 = forces_numpy(P, E, velY, SY, S2Y, geo, noise.astype(np.float64), curl.astype(np.float64))
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
