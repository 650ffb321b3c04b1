"""A second, independent restatement of the simulation step (src/sim.js) in numpy, FP64, written from the
WGSL separately from the C++ oracle.  Test infrastructure only: the oracle unit tests hold the oracle's
FP64 mode to these functions stage by stage and for a whole step.

Arrays are (nz, ny, nx[, 4]), x fastest like the reference's textures; P is the 64-float parameter block in
SIM_FIELDS order, E the extension block (soot age gate at E[0], E[1])."""
import numpy as np

import fire_sim as F

IDX = {n: i for i, n in enumerate(F.SIM_FIELDS)}


def par(P, name):
    return float(P[IDX[name]])


def smoothstep(e0, e1, x):
    t = np.clip((x - e0) / (e1 - e0), 0.0, 1.0)
    return t * t * (3.0 - 2.0 * t)


def mix(a, b, t):
    return a * (1.0 - t) + b * t


def grid(shape):
    nz, ny, nx = shape[:3]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return i, j, k


def trilinear(f, c):
    """textureSampleLevel with a linear, clamp-to-edge sampler at positions c (..., 3) in cell units."""
    nz, ny, nx = f.shape[:3]
    u = c - 0.5
    i0 = np.floor(u).astype(np.int64)
    fr = u - i0
    out = np.zeros(c.shape[:-1] + (f.shape[-1],))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = ((fr[..., 0] if dx else 1 - fr[..., 0]) * (fr[..., 1] if dy else 1 - fr[..., 1]) *
                     (fr[..., 2] if dz else 1 - fr[..., 2]))
                ix = np.clip(i0[..., 0] + dx, 0, nx - 1)
                iy = np.clip(i0[..., 1] + dy, 0, ny - 1)
                iz = np.clip(i0[..., 2] + dz, 0, nz - 1)
                out += w[..., None] * f[iz, iy, ix]
    return out


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
    """textureLoad at the clamped neighbour (i + di, j + dj, k + dk) of every cell (src/sim.js:114)."""
    nz, ny, nx = f.shape[:3]
    i, j, k = grid(f.shape)
    return f[np.clip(k + dk, 0, nz - 1), np.clip(j + dj, 0, ny - 1), np.clip(i + di, 0, nx - 1)]


def centres(shape):
    i, j, k = grid(shape)
    return np.stack([i, j, k], -1) + 0.5


def backtrace(vel, c, dt, dx):
    """src/sim.js:129-135: RK2 midpoint back-trace in cell units."""
    mid = c - 0.5 * dt * trilinear(vel, c)[..., :3] / dx
    return c - dt * trilinear(vel, mid)[..., :3] / dx


def outside_fade(b, dims):
    nx, ny, nz = dims
    lo = np.minimum(b[..., 0], b[..., 2])
    hi = np.maximum(b[..., 0] - nx, np.maximum(b[..., 1] - ny, b[..., 2] - nz))
    return np.clip(1.0 - np.maximum(-lo, hi), 0.0, 1.0)


def adv1(P, vel, S, S2):
    """src/sim.js:142-157 -> (velX, SX, S2X)."""
    nz, ny, nx = S.shape[:3]
    dt, dx = par(P, "dt"), par(P, "dx")
    c = centres(S.shape)
    b = backtrace(vel, c, dt, dx)
    fade = outside_fade(b, (nx, ny, nz))[..., None]
    ws = smoothstep(0.03, 0.4, b[..., 1] * dx)
    wind = np.stack([par(P, "windX") * ws, 0.0 * ws, par(P, "windZ") * ws], -1)
    velX = np.zeros(vel.shape)
    velX[..., :3] = mix(wind, trilinear(vel, b)[..., :3], fade)
    return velX, trilinear(S, b) * fade, trilinear(S2, b) * fade


def adv2(P, vel, S, S2, velX, SX, S2X):
    """src/sim.js:159-197 -> (velY, SY, S2Y)."""
    nz, ny, nx = S.shape[:3]
    dt, dx = par(P, "dt"), par(P, "dx")
    c = centres(S.shape)
    fw = c + dt * vel[..., :3] / dx
    b = backtrace(vel, c, dt, dx) - 0.5
    b0 = np.floor(b).astype(np.int64)
    revert = outside_fade(b + 0.5, (nx, ny, nz)) < 1.0
    outs = []
    for f, h, ch in ((vel, velX, 3), (S, SX, 4), (S2, S2X, 4)):
        N = h + 0.5 * (f - trilinear(h, fw))
        N[revert] = h[revert]
        mn = np.full(f.shape, 1e9)
        mx = np.full(f.shape, -1e9)
        for q in range(8):
            qx = np.clip(b0[..., 0] + (q & 1), 0, nx - 1)
            qy = np.clip(b0[..., 1] + ((q >> 1) & 1), 0, ny - 1)
            qz = np.clip(b0[..., 2] + ((q >> 2) & 1), 0, nz - 1)
            t = f[qz, qy, qx]
            mn, mx = np.minimum(mn, t), np.maximum(mx, t)
        out = np.minimum(np.maximum(N, np.minimum(mn, h)), np.maximum(mx, h))
        if ch == 3:
            out[..., 3] = 0.0
        else:
            out = np.maximum(out, 0.0)
        outs.append(out)
    return tuple(outs)


def curl_field(vel):
    """src/sim.js:200-211: half central-difference curl of the clamped neighbours, |w| in w."""
    L, R = ld(vel, -1, 0, 0), ld(vel, 1, 0, 0)
    B, T = ld(vel, 0, -1, 0), ld(vel, 0, 1, 0)
    K, Fw = ld(vel, 0, 0, -1), ld(vel, 0, 0, 1)
    w = np.stack([(T[..., 2] - B[..., 2]) - (Fw[..., 1] - K[..., 1]),
                  (Fw[..., 0] - K[..., 0]) - (R[..., 2] - L[..., 2]),
                  (R[..., 1] - L[..., 1]) - (T[..., 0] - B[..., 0])], -1) * 0.5
    return np.concatenate([w, np.linalg.norm(w, axis=-1)[..., None]], -1)


def div(P, velX):
    """src/sim.js:399-413 -> level-0 b."""
    dx = par(P, "dx")
    L, R = ld(velX, -1, 0, 0)[..., 0], ld(velX, 1, 0, 0)[..., 0]
    B, T = ld(velX, 0, -1, 0)[..., 1].copy(), ld(velX, 0, 1, 0)[..., 1]
    K, Fw = ld(velX, 0, 0, -1)[..., 2], ld(velX, 0, 0, 1)[..., 2]
    B[:, 0, :] = -velX[:, 0, :, 1]
    return ((R - L) + (T - B) + (Fw - K)) / (2.0 * dx) - velX[..., 3]


def neighbours(p):
    """The six neighbour values of every cell with the pressure ghosts: -p beyond the open sides and the top,
    +p below the floor (src/sim.js:447-451)."""
    nz, ny, nx = p.shape
    i, j, k = grid(p.shape)
    get = lambda a, b, c: p[np.clip(a, 0, nz - 1), np.clip(b, 0, ny - 1), np.clip(c, 0, nx - 1)]
    xm = np.where(i > 0, get(k, j, i - 1), -p)
    xp = np.where(i < nx - 1, get(k, j, i + 1), -p)
    zm = np.where(k > 0, get(k - 1, j, i), -p)
    zp = np.where(k < nz - 1, get(k + 1, j, i), -p)
    ym = np.where(j > 0, get(k, j - 1, i), p)
    yp = np.where(j < ny - 1, get(k, j + 1, i), -p)
    return xm, xp, ym, yp, zm, zp


def project(P, velX, p, geo):
    """src/sim.js:526-550 -> vel."""
    dx = par(P, "dx")
    xm, xp, ym, yp, zm, zp = neighbours(p)
    g = np.stack([xp - xm, yp - ym, zp - zm], -1) / (2.0 * dx)
    v = velX[..., :3] - g
    v[geo[..., 2] > 0.5] = 0.0
    v[:, 0, :, 1] = np.maximum(v[:, 0, :, 1], 0.0)
    vl = np.linalg.norm(v, axis=-1)
    cap = vl > 20.0
    v[cap] *= (20.0 / vl[cap])[:, None]
    out = np.zeros(velX.shape)
    out[..., :3] = v
    return out


def smooth_colour(p, b, h, colour):
    """One red-black colour sweep (src/sim.js:417-437): the cells with (x + y + z + colour) even."""
    nz, ny, nx = p.shape
    i, j, k = grid(p.shape)
    nb = neighbours(p)
    inside = [i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1]
    ssum = sum(np.where(m, v, 0.0) for m, v in zip(inside, nb))
    diag = 6.0 + (i == 0) + (i == nx - 1) + (k == 0) + (k == nz - 1) + (j == ny - 1) - (j == 0)
    return np.where((i + j + k + colour) % 2 == 0, (ssum - h * h * b) / diag, p)


def restrict(p, b, h, cdims):
    """src/sim.js:439-466: the 8-child mean of the residual."""
    cx, cy, cz = cdims
    xm, xp, ym, yp, zm, zp = neighbours(p)
    r = b - (xm + xp + ym + yp + zm + zp - 6.0 * p) / (h * h)
    return r[:2 * cz, :2 * cy, :2 * cx].reshape(cz, 2, cy, 2, cx, 2).mean(axis=(1, 3, 5))


def prolong_add(p, pc):
    """src/sim.js:468-495: trilinear prolongation with mirror ghosts (odd on the sides and top)."""
    nz, ny, nx = p.shape
    cz, cy, cx = pc.shape
    i, j, k = grid(p.shape)
    g = (np.stack([i, j, k], -1) + 0.5) * 0.5 - 0.5
    g0 = np.floor(g).astype(np.int64)
    f = g - g0
    nc = np.array([cx, cy, cz])
    acc = np.zeros(p.shape)
    for q8 in range(8):
        o = np.array([q8 & 1, (q8 >> 1) & 1, (q8 >> 2) & 1])
        q = g0 + o
        qc = np.clip(q, 0, nc - 1)
        val = pc[qc[..., 2], qc[..., 1], qc[..., 0]]
        val = np.where((q[..., 0] < 0) | (q[..., 0] >= cx), -val, val)
        val = np.where((q[..., 2] < 0) | (q[..., 2] >= cz), -val, val)
        val = np.where(q[..., 1] >= cy, -val, val)
        w = np.where(o == 1, f, 1.0 - f)
        acc += val * w[..., 0] * w[..., 1] * w[..., 2]
    return p + acc


def sweeps(p, b, h, n):
    for _ in range(n):
        p = smooth_colour(smooth_colour(p, b, h, 0), b, h, 1)
    return p


def vcycle(levels, coarse_iters, p0, b0, pre=2, post=2):
    """src/sim.js:588-599 on levels [(dims, h), ...]; returns the new level-0 p."""
    P, B = [p0], [b0]
    n = len(levels)
    for l in range(n - 1):
        P[l] = sweeps(P[l], B[l], levels[l][1], pre)
        B.append(restrict(P[l], B[l], levels[l][1], levels[l + 1][0]))
        cx, cy, cz = levels[l + 1][0]
        P.append(np.zeros((cz, cy, cx)))
    P[n - 1] = sweeps(P[n - 1], B[n - 1], levels[n - 1][1], coarse_iters)
    for l in range(n - 2, -1, -1):
        P[l] = sweeps(prolong_add(P[l], P[l + 1]), B[l], levels[l][1], post)
    return P[0]


def forces(P, E, velY, SY, S2Y, geo, noise, curl):
    """src/sim.js:214-396 (the vorticity of velY computed as the curl pass does) -> (velX, S, S2)."""
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


def step(P, E, state, geo, noise, curl, levels, coarse_iters, vcycles):
    """FireSim.step (src/sim.js:627-648) without the geometry rebuild: adv1, adv2, curl + forces, div,
    `vcycles` V(2,2) cycles warm-started from the level-0 p in `state`, project.  Returns the new state."""
    velX, SX, S2X = adv1(P, state["vel"], state["S"], state["S2"])
    velY, SY, S2Y = adv2(P, state["vel"], state["S"], state["S2"], velX, SX, S2X)
    velX, S, S2 = forces(P, E, velY, SY, S2Y, geo, noise, curl)
    b0 = div(P, velX)
    p = state["p"]
    for _ in range(vcycles):
        p = vcycle(levels, coarse_iters, p, b0)
    return {"vel": project(P, velX, p, geo), "S": S, "S2": S2, "velX": velX, "p": p}
