"""Discrete adjoint of the step (fire_adjoint.cu).

* Each stage's reverse kernel against central differences of the FP64 oracle's stage: for random seeded
  cotangents w of the outputs and directions v of the inputs, <w, (y(u + h v) - y(u - h v)) / 2h> must equal
  <J^T w, v> from the GPU adjoint (the dot-product identity, with the tangent taken by FP64 differences).
* The pressure solve's adjoint is the solve itself: symmetric to FP32 accuracy.
* The rollout's tape forward reproduces fire_sim_step bit for bit, and the backward leaves the simulation
  where the forward left it.
* Whole-rollout gradients (spot fluxes and the initial velocity) against FP64 central differences of the
  oracle's rollout, through checkpointed segments.

The forward map is continuous almost everywhere but not everywhere: the MacCormack limiter picks its 8-texel
stencil with floor() of the back-traced position and reverts to the plain advection outside the domain, so
an input direction that moves a back-trace across a cell boundary makes the output jump.  A central
difference that straddles such a jump is off by jump / 2h, and the chance of straddling one grows like h:
the expected error does not shrink with h, only the probability of meeting a jump does.  The differences
are therefore taken with a small step (FP64 keeps them accurate), where no cell's stencil changes; the
rollout test also reports the h = 1e-3 differences.
"""
import numpy as np
import pytest

import fire_cases as FC

DT = 1.0 / 120.0
H_STAGE = 1e-7     # central-difference step of the stage checks (inputs of order 1)
H_ROLL = 1e-9      # ... of the rollout checks (velocity in m/s; the state is of order 1)


def _smooth(shape, rng, w_zero=False):
    a = FC.smooth_noise(shape[:3], rng)
    if len(shape) == 4:
        a = np.stack([FC.smooth_noise(shape[:3], rng) for _ in range(shape[3])], -1)
        if w_zero:
            a[..., 3] = 0.0
    return a


def _clean_state(res, seed):
    """A random mid-burn state with every scalar strictly positive, so no input sits exactly on a
    max(., 0) kink (where a central difference averages the two one-sided slopes)."""
    st = FC.random_state(res, seed)
    for k in ("S", "S2", "SY", "S2Y", "SX", "S2X"):
        st[k] = (np.abs(st[k]) + 1e-3).astype(np.float32)
    return st


def _trilinear(f, pos):
    """Clamp-to-edge trilinear sample in cell units (texel i's centre at i + 0.5); f is (nz, ny, nx, C),
    pos (..., 3) in x, y, z order."""
    nz, ny, nx = f.shape[:3]
    idx, wts = [], []
    for a, n in enumerate((nx, ny, nz)):
        u = np.clip(pos[..., a] - 0.5, -1.0, float(n))
        i = np.floor(u)
        fr = u - i
        i = i.astype(np.int64)
        idx.append((np.clip(i, 0, n - 1), np.clip(i + 1, 0, n - 1)))
        wts.append((1.0 - fr, fr))
    out = 0.0
    for qx in (0, 1):
        for qy in (0, 1):
            for qz in (0, 1):
                w = wts[0][qx] * wts[1][qy] * wts[2][qz]
                out = out + w[..., None] * f[idx[2][qz], idx[1][qy], idx[0][qx]]
    return out


def _adv2_margins(st, dt, dx):
    """Per cell, how far adv2's discrete and piecewise choices are from switching: (1) in cells, the floor()
    of the limiter stencil's origin and the revert outside the domain; (2) in value, the gaps between the
    stencil's extreme texel and the next distinct texel, between those extremes and the own hat, and between
    the corrected value and the limiter bounds (the FP32 forward and the FP64 oracle may break a near-tie
    differently)."""
    vel = st["vel"].astype(np.float64)
    nz, ny, nx = vel.shape[:3]
    dims = (nx, ny, nz)
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    c = np.stack([xx + 0.5, yy + 0.5, zz + 0.5], -1)
    v = vel[..., :3]
    mid = c - v * (0.5 * dt) / dx
    bt = c - _trilinear(vel, mid)[..., :3] * dt / dx
    b = bt - 0.5
    pos = np.full((nz, ny, nx), np.inf)
    b0 = []
    for a, n in enumerate(dims):
        inside = (b[..., a] > -2.0) & (b[..., a] < n + 1.0)
        pos = np.minimum(pos, np.where(inside, np.abs(b[..., a] - np.round(b[..., a])), np.inf))
        b0.append(np.floor(np.clip(b[..., a], -2.0, n + 1.0)).astype(np.int64))
    lo = np.minimum(bt[..., 0], bt[..., 2])
    hi = np.maximum(bt[..., 0] - nx, np.maximum(bt[..., 1] - ny, bt[..., 2] - nz))
    out_m = np.maximum(-lo, hi)
    pos = np.minimum(pos, np.abs(out_m))
    revert = out_m > 0
    fw = c + v * dt / dx
    qi = [[np.clip(b0[a] + ((q >> a) & 1), 0, dims[a] - 1) for a in range(3)] for q in range(8)]
    idx = np.stack([(q[2] * ny + q[1]) * nx + q[0] for q in qi])
    val = np.full((nz, ny, nx), np.inf)
    for field, hat, nch in (("vel", "velX", 3), ("S", "SX", 4), ("S2", "S2X", 4)):
        Fv = st[field].astype(np.float64)
        Hv = st[hat].astype(np.float64)
        H = Hv[..., :nch]
        x = np.where(revert[..., None], H, H + (Fv[..., :nch] - _trilinear(Hv, fw)[..., :nch]) * 0.5)
        vals = np.stack([Fv[q[2], q[1], q[0]][..., :nch] for q in qi])
        for sgn in (1.0, -1.0):   # the minimum, then the maximum (as a minimum of negated values)
            sv = sgn * vals
            am = sv.argmin(0)
            ext = np.take_along_axis(sv, am[None], 0)[0]
            same = idx[..., None] == np.take_along_axis(np.broadcast_to(idx[..., None], sv.shape), am[None], 0)
            nxt = np.where(same, np.inf, sv).min(0)
            val = np.minimum(val, (nxt - ext).min(-1))
            val = np.minimum(val, np.abs(sgn * ext - H).min(-1))
        lo_b = np.minimum(vals.min(0), H)
        hi_b = np.maximum(vals.max(0), H)
        gap = np.minimum(np.abs(x - lo_b), np.abs(x - hi_b))
        val = np.minimum(val, np.where(revert[..., None], np.inf, gap).min(-1))
    return pos, val


@pytest.fixture(scope="module")
def campfire():
    import fire_sim as F
    return F.build_campfire(7)


# ------------------------------------------------------------------------------------------------ stages
# stage -> (oracle stages, inputs {sim field: adjoint buffer}, outputs {sim field: adjoint buffer});
# "lvl_p" / "lvl_b" stand for level 0's pressure / right-hand side.
STAGES = {
    "adv1": (["adv1"], {"vel": "vel", "S": "S", "S2": "S2"}, {"velX": "velX", "SX": "SX", "S2X": "S2X"}),
    "adv2": (["adv2"], {"vel": "vel", "S": "S", "S2": "S2", "velX": "velX", "SX": "SX", "S2X": "S2X"},
             {"velY": "velY", "SY": "SY", "S2Y": "S2Y"}),
    "forces": (["curl", "forces"], {"velY": "velY", "SY": "SY", "S2Y": "S2Y"}, {"velX": "F", "S": "S", "S2": "S2"}),
    "div": (["div"], {"velX": "F"}, {"lvl_b": "b"}),
    "project": (["project"], {"velX": "F", "lvl_p": "p"}, {"vel": "vel"}),
}


def _oracle_get(orc, name):
    if name == "lvl_p":
        return orc.get_level(0, "p", np.float64)
    if name == "lvl_b":
        return orc.get_level(0, "b", np.float64)
    return orc.get(name, np.float64)


def _oracle_put(orc, name, arr):
    if name == "lvl_p":
        orc.put_level(0, "p", arr)
    elif name == "lvl_b":
        orc.put_level(0, "b", arr)
    else:
        orc.put(name, arr)


@pytest.mark.gpu
@pytest.mark.parametrize("stage", list(STAGES))
def test_stage_adjoint_vs_fp64_differences(oracle_mod, campfire, stage):
    import fire_sim as F
    cfg = FC.C1
    spots = F.make_spots(5, 4, 1.0, 4.0, 0.02, 0.12)
    sim, orc = FC.make_pair(cfg, logs=campfire, dbl=True, spots=spots, soot_age=(0.02, 0.06),
                            params={"vortEps": 0.3, "turbAmp": 0.2, "visc": 1.0, "lamAge": 0.02, "windX": 0.4})
    blk = FC.sync_block(sim, orc, DT)
    sim.run_stage("geo", DT)
    orc.put("geo", sim.download("geo").astype(np.float64))
    rng = np.random.default_rng(11)
    state = _clean_state(cfg["res"], seed=3)
    nx, ny, nz = cfg["res"]
    state["lvl_p"] = (0.02 * FC.smooth_noise((nz, ny, nx), rng)).astype(np.float32)
    for k, v in state.items():
        if k == "lvl_p":
            sim.set_level(0, "p", v)
        else:
            sim.upload(k, v)
        _oracle_put(orc, k, v.astype(np.float64))
    ostages, ins, outs = STAGES[stage]
    adj = F.Adjoint(sim, 1, 1)
    adj.clear()
    # output cells whose limiter choices sit within 1e-3 cells (positions) or 1e-5 (values) of switching are
    # left out (zero cotangent): there the FP32 forward the adjoint linearises and the FP64 differences may
    # take different branches
    keep = np.ones((nz, ny, nx), bool)
    if stage == "adv2":
        pos, val = _adv2_margins(state, float(np.float32(DT)), sim.dx)
        keep = (pos > 1e-3) & (val > 1e-5)
        assert keep.mean() > 0.9
    w = {}
    for name, buf in outs.items():
        shape = adj._shape(buf)
        w[name] = rng.standard_normal(shape).astype(np.float32)
        w[name][~keep] = 0.0
        adj.put(buf, w[name])
    adj.stage(stage, DT)
    sim.sync()
    grads = {name: adj.get(buf).astype(np.float64) for name, buf in ins.items()}
    base = {name: state[name].astype(np.float64) for name in ins}
    dirs = {name: _smooth(base[name].shape, rng) for name in ins}
    h = H_STAGE

    def run(sign, flux_delta=None):
        for name in ins:
            _oracle_put(orc, name, base[name] + sign * h * dirs[name])
        if flux_delta is not None:
            e = blk[64:].copy()
            for q in range(len(spots)):
                e[16 + 8 * q + 4] += sign * h * flux_delta[q]
            orc.set_ext(e)
        for s in ostages:
            orc.stage(s)
        out = {name: _oracle_get(orc, name) for name in outs}
        orc.set_ext(blk[64:])
        return out

    yp, ym = run(+1), run(-1)
    fd = sum(float(np.sum(w[n].astype(np.float64) * (yp[n] - ym[n]) / (2 * h))) for n in outs)
    ad = sum(float(np.sum(grads[n] * dirs[n])) for n in ins)
    print(f"{stage}: <w, J v> by FP64 differences {fd:.9e}, <J^T w, v> by the adjoint {ad:.9e}")
    # adv2: what remains after the masking is the FP32 forward's rounding of near-ties (~1e-4)
    assert abs(fd - ad) <= (3e-4 if stage == "adv2" else 1e-4) * max(abs(fd), abs(ad)), (stage, fd, ad)
    if stage == "forces":   # the spot-flux gradients of the same cotangent
        gs = adj.grad_spots(len(spots))
        assert np.abs(gs).max() > 0
        for name in ins:
            _oracle_put(orc, name, base[name])
        flux = np.array([s[4] for s in spots], np.float64)
        fdir = rng.standard_normal(len(spots))
        # the fluxes travel in the FP32 block: step between FP32-representable values
        fp = (flux + 1e-4 * fdir).astype(np.float32).astype(np.float64)
        fm = (flux - 1e-4 * fdir).astype(np.float32).astype(np.float64)
        ys = []
        for fl in (fp, fm):
            e = blk[64:].copy()
            for q in range(len(spots)):
                e[16 + 8 * q + 4] = fl[q]
            orc.set_ext(e)
            for s in ostages:
                orc.stage(s)
            ys.append({n: _oracle_get(orc, n) for n in outs})
        orc.set_ext(blk[64:])
        fd_f = sum(float(np.sum(w[n].astype(np.float64) * (ys[0][n] - ys[1][n]))) for n in outs)
        ad_f = float(gs @ (fp - fm))
        print(f"forces, spot fluxes: FP64 differences {fd_f:.9e}, adjoint {ad_f:.9e}")
        assert abs(fd_f - ad_f) <= 1e-3 * abs(fd_f), (fd_f, ad_f, gs)
    adj.close()
    sim.close()


@pytest.mark.gpu
def test_pressure_adjoint_is_symmetric():
    import fire_sim as F
    sim = F.FireSim(res=(32, 64, 32), size=(0.4, 0.8, 0.4), vcycles=4)
    adj = F.Adjoint(sim, 1, 1)
    rng = np.random.default_rng(4)
    r1, r2 = rng.standard_normal((2, 32, 64, 32)).astype(np.float32)
    xs = []
    for r in (r1, r2):
        adj.clear()
        adj.put("p", r)
        adj.stage("vcycle", DT, arg=30)
        xs.append(adj.get("b").astype(np.float64))
    a = float(np.sum(r2 * xs[0]))
    b = float(np.sum(r1 * xs[1]))
    assert abs(a - b) <= 1e-5 * max(abs(a), abs(b))
    adj.close()
    sim.close()


# ------------------------------------------------------------------------------------------------ rollouts
RES = (24, 48, 24)
SIZE = (0.3, 0.6, 0.3)
VCYC = 10   # near-exact solves: the adjoint treats the pressure solve as A^-1


def _burning_sim(F, spots, preroll=30, residual_driven=False):
    if residual_driven:   # the source-fit workload's solve: over-relaxed V(2,2) to 1e-5, at most 8 cycles
        sim = F.FireSim(res=RES, size=SIZE, vcycles=VCYC, mg_max_cycles=8, mg_tol=1e-5)
        sim.set_mg_omega(1.2)
    else:
        sim = F.FireSim(res=RES, size=SIZE, vcycles=VCYC)
    sim.set_params({"vortEps": 0.3, "turbAmp": 0.2})
    sim.set_soot_age(0.02, 0.06)
    sim.set_bed_gain(0.0)
    sim.set_spots(spots)
    sim.step(DT, preroll)
    sim.sync()
    return sim


@pytest.mark.gpu
@pytest.mark.parametrize("residual_driven", [False, True])
def test_tape_forward_matches_step_and_backward_restores(residual_driven):
    """The taped forward is the step bit for bit, with fixed cycles and with the residual-driven solve (same
    cycle counts: every solve of the tape counts its cycles from zero and tests as the step's graph does), and
    stepping on after a backward gives the same bits as a simulation that never ran one."""
    import fire_sim as F
    spots = F.make_spots(9, 4, 1.0, 4.0, 0.02, 0.08)
    a, b = _burning_sim(F, spots, residual_driven=residual_driven), _burning_sim(F, spots, residual_driven=residual_driven)
    c0 = a.info().total_cycles
    adj = F.Adjoint(a, 7, 3)
    adj.forward(DT)
    b.step(DT, 7)
    a.sync(); b.sync()
    for name in ("vel", "S", "S2"):
        assert np.array_equal(a.download(name), b.download(name)), name
    assert np.array_equal(a.level(0, "p"), b.level(0, "p"))
    assert a.info().time == b.info().time and a.info().frame == b.info().frame
    if residual_driven:
        ca, cb = a.info().total_cycles - c0, b.info().total_cycles - c0
        assert ca == cb and ca >= 7, (ca, cb)
    adj.seed(S=np.ones(RES[::-1] + (4,), np.float32))
    adj.backward()
    a.sync()
    a.step(DT, 2)
    b.step(DT, 2)
    a.sync(); b.sync()
    for name in ("vel", "S", "S2"):
        assert np.array_equal(a.download(name), b.download(name)), name
    adj.close(); a.close(); b.close()


def _oracle_rollout(O, sim, blocks, start, flux=None, spots=None, flux64=None):
    """FP64 oracle rollout from `start` over the given per-step blocks; returns the final vel, S, S2.
    flux: spot fluxes written into the (FP32) blocks; flux64: spot fluxes held in double instead."""
    orc = O.OracleSim(RES, sim.dx, dbl=True)
    if flux64 is not None:
        orc.set_flux64(flux64)
    orc.set_tables(sim.download("noise").astype(np.float32), sim.download("curl").astype(np.float32))
    orc.set_logs(np.zeros(0, np.float32))
    for k in ("vel", "S", "S2", "geo"):
        orc.put(k, start[k])
    orc.put_level(0, "p", start["p"])
    for blk in blocks:
        b = blk.copy()
        if flux is not None:
            for q in range(len(flux)):
                b[64 + 16 + 8 * q + 4] = flux[q]
        orc.set_params(b[:64])
        orc.set_ext(b[64:])
        orc.step_raw(False, VCYC)
    return {k: orc.get(k, np.float64) for k in ("vel", "S", "S2")}


def _blocks(sim, n):
    """The parameter blocks of the next n steps (time and frame advanced as fire_sim_step does)."""
    b0 = sim.peek_block(DT)
    t, fr = float(sim.info().time), int(sim.info().frame)
    out = []
    for _ in range(n):
        b = b0.copy()
        b[5], b[6] = np.float32(t), np.float32(fr)
        out.append(b)
        t += float(np.float32(DT))
        fr += 1
    return out


@pytest.mark.gpu
def test_rollout_gradients_vs_fp64_differences(oracle_mod):
    """Gradients through 8 steps in segments of 3, 3 and 2 (two recomputed from their checkpoints).  The
    directions are tangent to the bounds the forward enforces: the initial-velocity direction leaves v.y
    alone on the floor cells where projection clamped it to 0 (there a back-trace sits exactly on a stencil
    boundary), and the scalar direction is proportional to S (zero where S is exactly 0)."""
    import fire_sim as F
    O = oracle_mod
    n_steps, k = 8, 3
    spots = F.make_spots(9, 4, 1.0, 4.0, 0.02, 0.08)
    sim = _burning_sim(F, spots)
    start = {n: sim.download(n).astype(np.float64) for n in ("vel", "S", "S2", "geo")}
    start["p"] = sim.level(0, "p").astype(np.float64)
    blocks = _blocks(sim, n_steps)
    adj = F.Adjoint(sim, n_steps, k)
    adj.forward(DT)
    rng = np.random.default_rng(21)
    shape = RES[::-1] + (4,)
    lam = {n: rng.standard_normal(shape) for n in ("vel", "S", "S2")}
    lam["vel"][..., 3] = 0.0
    adj.seed(*[lam[n].astype(np.float32) for n in ("vel", "S", "S2")])
    adj.backward()
    sim.sync()
    g = {n: adj.get(n).astype(np.float64) for n in ("vel", "S")}
    g_flux = adj.grad_spots(len(spots))
    J = lambda y: sum(float(np.sum(lam[n] * y[n])) for n in ("vel", "S", "S2"))

    def fd_state(name, d, h):
        sp, sm = dict(start), dict(start)
        sp[name], sm[name] = start[name] + h * d, start[name] - h * d
        return (J(_oracle_rollout(O, sim, blocks, sp)) - J(_oracle_rollout(O, sim, blocks, sm))) / (2 * h)

    # dot-product identity on the initial state: <lam, J d> (FP64 differences) = <J^T lam, d> (adjoint).
    # Away from the faces the map is smooth and the two agree to FP32 rounding.  The full-domain directions
    # also meet the places where it is not differentiable and the adjoint's subgradient and a central
    # difference (the mean of the one-sided slopes) legitimately differ: cells next to the faces (stencil
    # revert, clamped samples) and runs of exactly equal values (the saturated cores of the spots set the
    # same fuel in neighbouring cells, so the limiter's min / max ties).  Those get a looser bound, and the
    # scalar direction is mostly a uniform scaling of S, which moves tied values together.
    inner = np.zeros(shape[:3], bool)
    inner[2:-2, 2:-2, 2:-2] = True
    dv = _smooth(shape, rng, w_zero=True)
    floor_clamped = start["vel"][:, 0, :, 1] == 0.0
    dv[:, 0, :, 1][floor_clamped] = 0.0
    dS = (1.0 + 0.2 * _smooth(shape, rng)) * start["S"]
    for name, d, fld, tol in (("vel (interior)", dv * inner[..., None], "vel", 1e-4), ("vel", dv, "vel", 3e-2),
                              ("S", dS, "S", 1e-2)):
        ad = float(np.sum(g[fld] * d))
        fd = fd_state(fld, d, H_ROLL)
        print(f"initial {name}: differences {fd:.9e} (h = {H_ROLL:g}), {fd_state(fld, d, 1e-3):.9e} (h = 1e-3); "
              f"adjoint {ad:.9e}")
        assert abs(fd - ad) <= tol * abs(fd), (name, fd, ad)

    # spot-flux gradients against central differences with h = 1e-3 g/s (the fluxes travel in the FP32
    # parameter block, so the step is taken between the FP32-rounded values)
    base = np.array([s[4] for s in spots], np.float64)
    for q in range(len(spots)):
        fp, fm = base.copy(), base.copy()
        fp[q] = np.float32(base[q] + 1e-3)
        fm[q] = np.float32(base[q] - 1e-3)
        fdq = (J(_oracle_rollout(O, sim, blocks, start, fp)) - J(_oracle_rollout(O, sim, blocks, start, fm))) / (fp[q] - fm[q])
        print(f"spot {q}: differences {fdq:.9e}; adjoint {g_flux[q]:.9e}")
        assert abs(fdq - g_flux[q]) <= 1e-2 * max(abs(fdq), 1e-2 * np.abs(g_flux).max()), (q, fdq, g_flux[q])
    adj.close()
    sim.close()


@pytest.mark.gpu
def test_rollout_gradients_30_steps_vs_fp64_differences(oracle_mod):
    """The same checks through 30 steps in three checkpointed segments of 10.  At this grid the FP32 forward
    and the FP64 oracle stay within 1e-5 of each other over 30 steps (test_horizon_of_fp64_checks), so a
    central difference of the FP64 oracle still describes the map the GPU adjoint differentiates, while the
    sensitivity to the initial state has grown about sevenfold from 8 steps."""
    import fire_sim as F
    O = oracle_mod
    n_steps, k = 30, 10
    spots = F.make_spots(9, 4, 1.0, 4.0, 0.02, 0.08)
    sim = _burning_sim(F, spots)
    start = {n: sim.download(n).astype(np.float64) for n in ("vel", "S", "S2", "geo")}
    start["p"] = sim.level(0, "p").astype(np.float64)
    blocks = _blocks(sim, n_steps)
    adj = F.Adjoint(sim, n_steps, k)
    adj.forward(DT)
    rng = np.random.default_rng(22)
    shape = RES[::-1] + (4,)
    lam = {n: rng.standard_normal(shape) for n in ("vel", "S", "S2")}
    lam["vel"][..., 3] = 0.0
    adj.seed(*[lam[n].astype(np.float32) for n in ("vel", "S", "S2")])
    adj.backward()
    sim.sync()
    g = {n: adj.get(n).astype(np.float64) for n in ("vel", "S")}
    g_flux = adj.grad_spots(len(spots))
    J = lambda y: sum(float(np.sum(lam[n] * y[n])) for n in ("vel", "S", "S2"))

    def fd_state(name, d, h):
        sp, sm = dict(start), dict(start)
        sp[name], sm[name] = start[name] + h * d, start[name] - h * d
        return (J(_oracle_rollout(O, sim, blocks, sp)) - J(_oracle_rollout(O, sim, blocks, sm))) / (2 * h)

    inner = np.zeros(shape[:3], bool)
    inner[2:-2, 2:-2, 2:-2] = True
    dv = _smooth(shape, rng, w_zero=True)
    floor_clamped = start["vel"][:, 0, :, 1] == 0.0
    dv[:, 0, :, 1][floor_clamped] = 0.0
    dS = (1.0 + 0.2 * _smooth(shape, rng)) * start["S"]
    for name, d, fld, tol in (("vel (interior)", dv * inner[..., None], "vel", 1e-3), ("vel", dv, "vel", 5e-2),
                              ("S", dS, "S", 2e-2)):
        ad = float(np.sum(g[fld] * d))
        fd = fd_state(fld, d, H_ROLL)
        print(f"30 steps, initial {name}: differences {fd:.9e} (h = {H_ROLL:g}); adjoint {ad:.9e}; rel {abs(fd - ad) / abs(fd):.2e}")
        assert abs(fd - ad) <= tol * abs(fd), (name, fd, ad)
    # spot fluxes: over 30 steps a difference step of 1e-3 g/s (the FP32 block's resolution allows no less)
    # straddles limiter jumps, so the oracle holds the fluxes in double and the step is 1e-7 g/s
    base = np.array([s[4] for s in spots], np.float64)
    hq = 1e-7
    for q in range(len(spots)):
        fp, fm = base.copy(), base.copy()
        fp[q] += hq
        fm[q] -= hq
        fdq = (J(_oracle_rollout(O, sim, blocks, start, flux64=fp)) - J(_oracle_rollout(O, sim, blocks, start, flux64=fm))) / (2 * hq)
        print(f"30 steps, spot {q}: differences {fdq:.9e} (h = {hq:g} g/s); adjoint {g_flux[q]:.9e}")
        assert abs(fdq - g_flux[q]) <= 1e-2 * max(abs(fdq), 1e-2 * np.abs(g_flux).max()), (q, fdq, g_flux[q])
    adj.close()
    sim.close()


def test_horizon_of_fp64_checks(oracle_mod):
    """Why the rollout gradient is checked against FP64 differences at 8 and 30 steps and not at the 120 of
    the source-fit workload, on the oracle alone (24x48x24, the rollout tests' burning state): the FP32 and
    FP64 trajectories from one state agree to 1e-4 through 30 steps but separate by more than 1e-2 by 120
    steps, because the flow amplifies perturbations (the FP64 response to a 1e-9 change of the initial
    velocity grows by more than 1e4 between 8 and 120 steps).  FP32 rounding alone moves the 120-step state
    as far as any finite difference would probe: the discrete gradient there is that of a chaotic map."""
    O = oracle_mod
    O.set_threads(O.lib().orc_num_threads())
    dx = np.float32(np.float64(np.float32(SIZE[0])) / RES[0])
    noise = O.noise_table(128, 1)
    curl = O.curl_table(noise)
    spots = O.make_spots(9, 4, 1.0, 4.0, 0.02, 0.08)

    def block(t, f):
        b = np.zeros(208, np.float32)
        b[:64] = O.sim_defaults()
        b[0], b[1], b[2] = RES
        b[3], b[4], b[5], b[6] = dx, np.float32(DT), np.float32(t), f
        b[8] = b[10] = np.float32(-np.float32(SIZE[0]) / np.float32(2))
        b[34], b[35] = 0.3, 0.2          # vortEps, turbAmp
        e = b[64:]
        e[0], e[1], e[2], e[3], e[4] = 0.02, 0.06, 0.0, len(spots), 4.0
        for i, sp in enumerate(spots):
            e[16 + 8 * i: 16 + 8 * i + 5] = sp
        return b

    def make(dbl):
        o = O.OracleSim(RES, float(dx), dbl=dbl)
        o.set_tables(noise, curl)
        o.set_logs(np.zeros(0, np.float32))
        return o

    o, t = make(False), 0.0
    for s in range(30):
        b = block(t, s)
        o.set_params(b[:64]); o.set_ext(b[64:]); o.step_raw(s == 0, VCYC)
        t += float(np.float32(DT))
    start = {k: o.get(k) for k in ("vel", "S", "S2", "geo")}
    p0 = o.get_level(0, "p")

    def run(dbl, n, dvel=None):
        r = make(dbl)
        for k, v in start.items():
            r.put(k, v.astype(np.float64) if dbl else v)
        if dvel is not None:
            r.put("vel", start["vel"].astype(np.float64) + dvel)
        r.put_level(0, "p", p0.astype(np.float64) if dbl else p0)
        tt = t
        for s in range(n):
            b = block(tt, 30 + s)
            r.set_params(b[:64]); r.set_ext(b[64:]); r.step_raw(False, VCYC)
            tt += float(np.float32(DT))
        return np.concatenate([r.get(k, np.float64).ravel() for k in ("vel", "S", "S2")])

    sep = {n: np.linalg.norm(run(False, n) - run(True, n)) / np.linalg.norm(run(True, n)) for n in (30, 120)}
    d = np.random.default_rng(3).standard_normal(start["vel"].shape)
    d[..., 3] = 0.0
    amp = {n: np.linalg.norm(run(True, n, 1e-9 * d) - run(True, n)) / (1e-9 * np.linalg.norm(d)) for n in (8, 120)}
    print(f"\nFP32 vs FP64 separation: 30 steps {sep[30]:.2e}, 120 steps {sep[120]:.2e}; "
          f"FP64 sensitivity: 8 steps {amp[8]:.3e}, 120 steps {amp[120]:.3e}")
    assert sep[30] < 1e-4 and sep[120] > 1e-2, sep
    assert amp[120] > 1e4 * amp[8], amp


@pytest.mark.gpu
def test_loss_and_autograd_contract():
    import torch
    import fire_sim as F
    spots = F.make_spots(9, 4, 1.0, 4.0, 0.02, 0.08)
    sim = _burning_sim(F, spots)
    adj = F.Adjoint(sim, 5, 2)
    vel0, S0, S20 = (torch.from_numpy(sim.download(n).astype(np.float32)) for n in ("vel", "S", "S2"))
    target = sim.download("S").astype(np.float32) * 0.9
    # the loss entry point against the same sum in numpy
    adj.forward(DT)
    L = adj.loss(target)
    S = sim.download("S").astype(np.float64)
    want = np.sum((1000.0 * (S[..., 0] - target[..., 0])) ** 2 + (S[..., 2] - target[..., 2]) ** 2)
    assert L == pytest.approx(want, rel=1e-6)
    # autograd.Function contract: the same rollout through FireRollout, then backward of a scalar
    Roll = F.rollout_function()
    flux = torch.tensor([s[4] for s in spots], dtype=torch.float64, requires_grad=True)
    v0 = vel0.clone().requires_grad_(True)
    vel, S1, S21 = Roll.apply(adj, DT, spots, v0, S0.clone(), S20.clone(), flux)
    tgt = torch.from_numpy(target)
    loss = ((1000.0 * (S1[..., 0] - tgt[..., 0])) ** 2).sum() + ((S1[..., 2] - tgt[..., 2]) ** 2).sum()
    loss.backward()
    assert v0.grad is not None and flux.grad is not None
    assert torch.isfinite(v0.grad).all() and torch.isfinite(flux.grad).all()
    assert float(flux.grad.abs().max()) > 0
    adj.close()
    sim.close()
