"""Ensembles (fire_ensemble_*): members of different grids stepped by batched launches must give the fields
each member gives when stepped alone.  The batched kernels run the same kernel bodies; the first step is
bit-identical, later steps agree to FP32 rounding (the compiler may contract a*b+c into FMA differently in
the batched and per-simulation instantiations), so the bound is relative L2 1e-4 after 6 steps."""
import numpy as np
import pytest

import fire_cases as FC

pytestmark = pytest.mark.gpu

# grids chosen to cover every batched path: levels outside the tail (48x96x48: two; 64x128x64: two), the
# single-CTA tail (48x96x48 from level 2, 24x48x24 from level 1) and the cluster tail (32x64x32 from level 1,
# 64x128x64 from level 2)
MEMBERS = [
    dict(res=(48, 96, 48), size=(0.6, 1.2, 0.6), seed=11, spots=5),
    dict(res=(32, 64, 32), size=(0.4, 0.8, 0.4), seed=12, spots=2),
    dict(res=(24, 48, 24), size=(0.3, 0.6, 0.3), seed=13, spots=3),
    dict(res=(64, 128, 64), size=(0.8, 1.6, 0.8), seed=14, spots=8),
    dict(res=(32, 64, 32), size=(0.4, 0.8, 0.4), seed=15, spots=4),
]
DT = 1.0 / 120.0


def _configure(sim, m):
    import fire_sim as F
    sim.set_spots(F.make_spots(m["seed"], m["spots"], 1.0, 4.0, 0.0125 * 1.6, 0.3 * m["size"][0]))
    sim.set_params({"seed": float(m["seed"]), "vortEps": 0.3, "turbAmp": 0.2})
    sim.set_soot_age(0.02, 0.06)
    sim.set_bed_gain(0.0)


def test_ensemble_equals_members_alone():
    import fire_sim as F
    ens = F.Ensemble(MEMBERS, vcycles=4)
    for sim, m in zip(ens.members, MEMBERS):
        _configure(sim, m)
    alone = []
    for m in MEMBERS:
        s = F.FireSim(res=m["res"], size=m["size"], vcycles=4)
        _configure(s, m)
        alone.append(s)
    ens.step(DT, 1)
    ens.sync()
    for s in alone:
        s.step(DT, 1)
        s.sync()
    for k, (a, b) in enumerate(zip(ens.members, alone)):   # one step from rest: bit-identical
        for name in ("vel", "S", "S2"):
            assert np.array_equal(a.download(name), b.download(name)), (k, name)
    ens.step(DT, 5)
    ens.sync()
    for s in alone:
        s.step(DT, 5)
        s.sync()
    for k, (a, b) in enumerate(zip(ens.members, alone)):
        for name in ("vel", "S", "S2"):
            x, y = a.download(name), b.download(name)
            assert np.isfinite(x).all()
            assert FC.rel_l2(x, y) < 1e-4, (k, name, FC.rel_l2(x, y))
        assert FC.rel_l2(a.level(0, "p"), b.level(0, "p")) < 1e-4, k
        assert a.info().frame == b.info().frame == 6
    # the fire has started in every member
    assert all(float(m.download("S")[..., 0].max()) > 0.05 for m in ens.members)
    for s in alone:
        s.close()
    ens.close()


@pytest.mark.parametrize("member", [0, 3])
def test_ensemble_member_step_vs_oracle(oracle_mod, member):
    """A member of a batched ensemble against the oracle directly: after 10 batched steps (a developed fire),
    the member's state goes into the FP32 oracle with the member's own parameter block for the next step,
    and one more batched step must match one oracle step at the one-step tolerance of tests/test_gpu_step.py
    (1e-3 relative + 1e-4 of each channel's scale, at most 0.5 % of cells beyond)."""
    import fire_sim as F
    ens = F.Ensemble(MEMBERS, vcycles=4)
    for sim, m in zip(ens.members, MEMBERS):
        _configure(sim, m)
    ens.step(DT, 10)
    ens.sync()
    sim = ens.members[member]
    m = MEMBERS[member]
    orc = oracle_mod.OracleSim(m["res"], sim.dx)
    orc.set_tables(sim.download("noise").astype(np.float32), sim.download("curl").astype(np.float32))
    orc.set_logs(np.zeros(0, np.float32))
    for name in ("vel", "S", "S2", "geo"):
        orc.put(name, sim.download(name))
    orc.put_level(0, "p", sim.level(0, "p"))
    FC.sync_block(sim, orc, DT)
    ens.step(DT, 1)
    ens.sync()
    orc.step_raw(False, 4)
    assert float(sim.download("S")[..., 0].max()) > 0.05
    for name in ("vel", "S", "S2"):
        g, o = sim.download(name), orc.get(name)
        for c in range(4):
            FC.compare(g[..., c], o[..., c], 1e-3, 1e-4, 5e-3, what=f"member {member} {name}[{c}]")
    FC.compare(sim.level(0, "p"), orc.get_level(0, "p"), 1e-3, 1e-4, 5e-3, what=f"member {member} p")
    ens.close()


def test_ensemble_rejects_bad_configs():
    import fire_sim as F
    with pytest.raises(F.FireError):
        F.Ensemble([dict(res=(32, 64, 32), size=(0.4, 0.8, 0.4))] * 65)
    with pytest.raises(F.FireError):
        F.Ensemble([])


def test_tile_candidates_agree_and_autotune_picks_one():
    """Every tile candidate of the batched stages computes the same per-cell arithmetic: after 10 steps with
    the default tiles, one more step with any candidate gives the default tiles' fields to FP32 rounding.
    The autotuner's step gives the same fields as a plain step and reports a valid choice with its timings."""
    import fire_sim as F
    members = MEMBERS[:3]

    def run(tiles=None, tune=False):
        ens = F.Ensemble(members, vcycles=4)
        ens.set_autotune(-1)
        for sim, m in zip(ens.members, members):
            _configure(sim, m)
        ens.step(DT, 10)
        if tiles is not None:
            ens.set_tiles(tiles)
        if tune:
            ens.set_autotune(0)
        ens.step(DT, 1)
        ens.sync()
        out = [{n: s.download(n) for n in ("vel", "S", "S2")} for s in ens.members]
        chosen = ens.tiles()
        ens.close()
        return out, chosen

    ref, _ = run()
    variants = [[v, v, min(v, 2), v, v] for v in range(1, 4)] + [[0, 0, 1, 0, 0], [0, 0, 2, 0, 0]]
    for tiles in variants + ["tune"]:
        got, chosen = run(tune=True) if tiles == "tune" else run(tiles)
        for k in range(len(members)):
            for n in ("vel", "S", "S2"):
                assert FC.rel_l2(got[k][n], ref[k][n]) < 1e-5, (tiles, k, n)
    tiles, ms = chosen
    assert all(0 <= t < (3 if i == 2 else 4) for i, t in enumerate(tiles))
    assert (ms[[0, 1, 3, 4]] > 0).all() and (ms[2, :3] > 0).all()
