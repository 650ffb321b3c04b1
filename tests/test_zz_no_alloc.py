"""The allocation-free pressure solve (fire_poisson_vcycles_noalloc) against the simulation's own V-cycle.

fire_poisson_vcycles_noalloc exists for callers that cannot allocate device memory at solve time (their
device memory belongs to another allocator, their frame budget is fixed, or they are recording a CUDA
graph): they pass their own level-0 arrays and the coarse levels live in a fixed device array inside the
library.  This test calls it through the C ABI, twice in a row on the same arrays, and checks each result
against the existing V-cycle path (fire_sim_run_stage with FIRE_STAGE_VCYCLE): both run the same kernels in
the same order on the same values, so the results must agree bit for bit.  The first result is also held to
the oracle's V-cycle at the V-cycle parity tolerance (1e-4 relative + 1e-5 of the field's scale), and the
timeout status query must report a clean run.  The file is named so that pytest collects it last; it does
not depend on any other test having run.
"""
import ctypes

import numpy as np
import pytest

import fire_cases as FC
import fire_sim as F

pytestmark = pytest.mark.gpu


def _field(shape, seed, scale):
    return (FC.smooth_noise(shape, np.random.default_rng(seed), 1) * scale).astype(np.float32)


@pytest.mark.parametrize("res", [(64, 128, 64), (48, 96, 48)])
def test_noalloc_vcycles_match_simulation_vcycles(oracle_mod, res):
    torch = pytest.importorskip("torch")
    lib = F.load_library()
    size = (0.005 * res[0], 0.005 * res[1], 0.005 * res[2])
    sim = F.FireSim(res=res, size=size, vcycles=1)
    shape = (res[2], res[1], res[0])
    p0 = _field(shape, 1, 0.01)
    b0 = _field(shape, 2, 50.0)
    sim.set_level(0, "p", p0)
    sim.set_level(0, "b", b0)
    orc = oracle_mod.OracleSim(res, sim.dx)
    orc.put_level(0, "p", p0)
    orc.put_level(0, "b", b0)
    orc.vcycle()

    p_dev = torch.from_numpy(p0.copy()).cuda()
    b_dev = torch.from_numpy(b0.copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    h = sim.levels[0]["h"]
    for call in range(2):
        rc = lib.fire_poisson_vcycles_noalloc(ctypes.c_void_p(p_dev.data_ptr()), ctypes.c_void_p(b_dev.data_ptr()),
                                              res[0], res[1], res[2], ctypes.c_float(h), 1, ctypes.c_void_p(stream))
        assert rc == 0, f"call {call}: status {rc}"
        assert lib.fire_poisson_noalloc_status(ctypes.c_void_p(stream)) == 0, f"call {call}: wait timeout reported"
        sim.run_stage("vcycle", 0.01)
        sim.sync()
        got = p_dev.cpu().numpy()
        np.testing.assert_array_equal(got, sim.level(0, "p"), err_msg=f"noalloc call {call}")
        if call == 0:
            FC.compare(got, orc.get_level(0, "p"), 1e-4, 1e-5, 0, what="noalloc vs oracle")
    # the right-hand side is read only
    np.testing.assert_array_equal(b_dev.cpu().numpy(), b0)
    sim.close()


def test_noalloc_rejects_grids_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    lib = F.load_library()
    p = torch.zeros(4, device="cuda")
    # a 512^3 level 0 needs ~153 MB of coarse levels, far beyond the fixed array: rejected before any work
    rc = lib.fire_poisson_vcycles_noalloc(ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(p.data_ptr()),
                                          512, 512, 512, ctypes.c_float(0.01), 1, None)
    assert rc == 1
