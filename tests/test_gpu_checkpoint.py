"""Checkpoint and resume (fire_sim_save / fire_sim_load): a simulation restored from a checkpoint continues
bit for bit as the saved one does — with logs and spots, a burst and a gust in progress at the checkpoint,
and the tolerance-driven over-relaxed solve, whose next-step cycle prediction travels in the checkpoint —
and a checkpoint of another grid, of the wrong length or with a corrupted header is refused."""
import numpy as np
import pytest

import fire_cases as FC
import fire_sim as F

pytestmark = pytest.mark.gpu

RES, SIZE, DT = (32, 64, 32), (0.4, 0.8, 0.4), 1.0 / 120.0


def _make():
    sim = F.FireSim(res=RES, size=SIZE, logs=F.build_campfire(7), vcycles=4, mg_max_cycles=8, mg_tol=1e-5)
    sim.set_mg_omega(1.2)
    sim.set_spots(F.make_spots(3, 3, 1.0, 4.0, 0.02, 0.1))
    return sim


def _state(sim):
    out = {k: sim.download(k) for k in ("vel", "S", "S2", "geo")}
    out["p"] = sim.level(0, "p")
    return out


def test_resume_is_bit_exact():
    a = _make()
    a.step(DT, 12)
    a.inject((0.02, 0.08, -0.03), 1.0, 0.05)   # a burst and a gust still running at the checkpoint
    a.gust(1.0, 0.2)
    a.step(DT, 3)
    a.sync()
    blob = a.save()
    a.step(DT, 10)
    a.sync()
    want, info_a = _state(a), a.info()
    b = _make()
    b.step(DT, 2)                            # a different state, overwritten by the load
    b.load(blob)
    b.step(DT, 10)
    b.sync()
    got, info_b = _state(b), b.info()
    for k in want:
        assert np.array_equal(got[k], want[k]), k
    assert info_b.time == info_a.time and info_b.frame == info_a.frame
    assert info_b.total_cycles == info_a.total_cycles and info_b.last_cycles == info_a.last_cycles
    assert float(want["S"][..., 0].max()) > 0.05
    a.close(); b.close()


def test_load_refuses_foreign_or_damaged_checkpoints():
    a = _make()
    a.step(DT, 2)
    blob = a.save()
    other = F.FireSim(res=(32, 64, 16), size=(0.4, 0.8, 0.2), vcycles=4)
    with pytest.raises(F.FireError) as e:
        other.load(blob)                     # another grid: the sizes differ
    assert e.value.code == 1
    with pytest.raises(F.FireError):
        a.load(blob[:-4])
    bad = bytearray(blob)
    bad[0] ^= 0xFF
    with pytest.raises(F.FireError):
        a.load(bytes(bad))
    before = _state(a)
    a.load(blob)                             # the intact checkpoint still loads
    assert all(np.array_equal(before[k], v) for k, v in _state(a).items() if k != "geo")
    a.close(); other.close()
