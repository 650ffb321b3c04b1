"""Error behaviour of the C ABI entry points beyond the step (status codes, no state change on a refused call),
as the reference's UniformStruct.set throws on an unknown name (src/gpu.js:65)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mg_omega_and_adjoint_misuse():
    import fire_sim as F
    sim = F.FireSim(res=(16, 32, 16), size=(0.2, 0.4, 0.2), vcycles=2)
    for bad in (0.0, -1.0, 2.0, float("nan")):
        with pytest.raises(F.FireError) as e:
            sim.set_mg_omega(bad)
        assert e.value.code == 1
    sim.set_mg_omega(1.2)
    sim.step(0.01, 2)
    sim.sync()
    adj = F.Adjoint(sim, 4, 2)
    with pytest.raises(F.FireError) as e:   # a backward needs a forward first
        adj.backward()
    assert e.value.code == 6
    with pytest.raises(F.FireError):
        adj.put("vel", np.zeros(10, np.float32))   # wrong size
    with pytest.raises(F.FireError):
        adj.stage("geo", 0.01)                     # no adjoint of the geometry stage
    with pytest.raises(F.FireError):
        F.Adjoint(sim, 0, 1)
    with pytest.raises(F.FireError):
        F.Adjoint(sim, 4, 0)
    adj.forward(0.01)
    adj.seed(S=np.ones((16, 32, 16, 4), np.float32))
    adj.backward()
    sim.sync()
    assert np.isfinite(adj.get("vel")).all()
    adj.close()
    sim.close()


def test_ensemble_tile_api_misuse():
    import fire_sim as F
    ens = F.Ensemble([dict(res=(16, 32, 16), size=(0.2, 0.4, 0.2))] * 2, vcycles=2)
    assert ens.tiles() is None                      # no tuning step yet
    for bad in ([0, 0, 3, 0, 0], [4, 0, 0, 0, 0], [0, 0, 0, 0, -1]):
        with pytest.raises(F.FireError):
            ens.set_tiles(bad)
    with pytest.raises(F.FireError):
        ens.set_autotune(-2)
    ens.set_tiles([1, 2, 1, 3, 0])
    tiles, _ = ens.tiles()
    assert list(tiles) == [1, 2, 1, 3, 0]
    ens.step(0.01, 2)
    ens.sync()
    assert all(np.isfinite(m.download("vel")).all() for m in ens.members)
    ens.close()


def test_study_variant_and_wait_limit_arguments():
    """fire_poisson_set_study applies to the FP32 form only and needs at least one coarsest sweep;
    fire_sim_set_tail_wait_limit refuses a negative bound."""
    import fire_sim as F
    ir = F.Poisson((16, 32, 16), 1.0, "ir32")
    with pytest.raises(F.FireError) as e:
        ir.set_study(30)
    assert e.value.code == 1
    ir.close()
    ps = F.Poisson((16, 32, 16), 1.0, "fp32")
    for bad in (0, -3):
        with pytest.raises(F.FireError):
            ps.set_study(bad)
    ps.set_study(16)
    ps.close()
    sim = F.FireSim(res=(16, 32, 16), size=(0.2, 0.4, 0.2), vcycles=2)
    with pytest.raises(F.FireError) as e:
        sim.set_tail_wait_limit(-1)
    assert e.value.code == 1
    sim.set_tail_wait_limit(1 << 22)
    sim.step(0.01, 1)
    sim.sync()
    sim.close()


def test_allocation_failure_is_reported_and_harmless():
    """A grid whose fields exceed device memory (1000 x 1000 x 2000 cells: ~350 GB of fields, within the
    32-bit cell-offset limit) fails at allocation with FIRE_ERR_OOM, and the device stays usable."""
    import fire_sim as F
    with pytest.raises(F.FireError) as e:
        F.FireSim(res=(1000, 1000, 2000), size=(1.0, 1.0, 2.0), vcycles=1)
    assert e.value.code == 5
    sim = F.FireSim(res=(16, 32, 16), size=(0.2, 0.4, 0.2), vcycles=2)
    sim.step(0.01, 2)
    sim.sync()
    assert np.isfinite(sim.download("vel")).all()
    sim.close()
