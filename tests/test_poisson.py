"""Standalone pressure Poisson solver (fire_poisson_*): the FP64 conjugate-gradient oracle pinned against a
dense solve, the seeded right-hand side against a numpy restatement, and the FP32 / FP16 / BF16 solvers
against the oracle (one V-cycle bit-for-bit in structure, solutions to tolerance, FP64-recomputed residual)."""
import math

import numpy as np
import pytest

import fire_cases as FC


def _pcg1(n):
    n = np.uint64(n)
    s = (n * np.uint64(747796405) + np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
    w = (((s >> ((s >> np.uint64(28)) + np.uint64(4))) ^ s) * np.uint64(277803737)) & np.uint64(0xFFFFFFFF)
    return int((w >> np.uint64(22)) ^ w)


def _rand2(n, m):
    return _pcg1((n ^ _pcg1(m)) & 0xFFFFFFFF) / 4294967295.0


def _sources_py(seed, n, res):
    """Source rows of fire_poisson_sources restated in Python doubles."""
    out = []
    for i in range(n):
        k = 6 * i
        u1 = max(_rand2(seed, k + 4), 1e-12)
        u2 = _rand2(seed, k + 5)
        out.append([_rand2(seed, k) * res[0], _rand2(seed, k + 1) * res[1], _rand2(seed, k + 2) * res[2],
                    1.0 + 3.0 * _rand2(seed, k + 3), math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)])
    return np.array(out, np.float32)


def _pcg3d_np(x, y, z):
    M = np.uint32
    v0 = x.astype(M) * M(1664525) + M(1013904223)
    v1 = y.astype(M) * M(1664525) + M(1013904223)
    v2 = z.astype(M) * M(1664525) + M(1013904223)
    v0 = v0 + v1 * v2; v1 = v1 + v2 * v0; v2 = v2 + v0 * v1
    v0 ^= v0 >> M(16); v1 ^= v1 >> M(16); v2 ^= v2 >> M(16)
    v0 = v0 + v1 * v2; v1 = v1 + v2 * v0; v2 = v2 + v0 * v1
    return v0, v1, v2


def _rhs_py(res, seed, n_sources, noise):
    nx, ny, nz = res
    src = _sources_py(seed, n_sources, res).astype(np.float64)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    px, py, pz = x + 0.5, y + 0.5, z + 0.5
    v = np.zeros((nz, ny, nx))
    for cx, cy, cz, sg, a in src:
        v += a * np.exp(-((px - cx) ** 2 + (py - cy) ** 2 + (pz - cz) ** 2) / (2 * sg * sg))
    with np.errstate(over="ignore"):
        h0, h1, _ = _pcg3d_np(x.astype(np.uint32), y.astype(np.uint32),
                              z.astype(np.uint32) ^ np.uint32((seed * 0x9E3779B9) & 0xFFFFFFFF))
    u1 = ((h0 >> np.uint32(8)).astype(np.float64) + 1.0) / 16777216.0
    u2 = (h1 >> np.uint32(8)).astype(np.float64) / 16777216.0
    v += noise * np.sqrt(-2.0 * np.log(u1)) * np.cos(2 * np.pi * u2)
    return v - v.mean()


# ------------------------------------------------------------------ CPU: the oracle and host logic
def test_cg_matches_dense_solve(oracle_mod):
    """The FP64 CG oracle solves the multigrid's operator: against numpy's dense solve on 6x8x6."""
    nx, ny, nz, h = 6, 8, 6, 0.01
    n = nx * ny * nz
    A = np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n); e[i] = 1.0
        A[:, i] = oracle_mod.pressure_apply(e.reshape(nz, ny, nx), h).ravel()
    np.testing.assert_allclose(A, A.T, rtol=0, atol=1e-9 * np.abs(A).max())
    assert np.linalg.eigvalsh(-A).min() > 0           # -A is symmetric positive definite
    b = np.random.default_rng(1).standard_normal(n)
    want = np.linalg.solve(A, b)
    x, it, rel = oracle_mod.pressure_cg(b.reshape(nz, ny, nx), h, tol=1e-13)
    assert rel <= 1e-13 and it <= n
    np.testing.assert_allclose(x.ravel(), want, rtol=0, atol=1e-10 * np.abs(want).max())


def test_operator_matches_vcycle_residual(oracle_mod):
    """orc_pressure_rel_residual uses the same operator as the multigrid's residual (src/sim.js:439-466)."""
    orc = oracle_mod.OracleSim((16, 32, 16), 0.01, dbl=True)
    rng = np.random.default_rng(2)
    p = rng.standard_normal((16, 32, 16)).astype(np.float32)
    b = rng.standard_normal((16, 32, 16)).astype(np.float32)
    orc.put_level(0, "p", p)
    orc.put_level(0, "b", b)
    rr, bb = orc.residual()
    h = float(np.float32(0.01))   # the level spacing is held in FP32
    assert oracle_mod.pressure_rel_residual(b, p, h) == pytest.approx(math.sqrt(rr / bb), rel=1e-12)


def test_poisson_sources_match_python(firelib):
    import fire_sim as F
    for seed, n, res in [(3, 32, (256, 512, 256)), (11, 5, (32, 64, 32))]:
        np.testing.assert_allclose(F.poisson_sources(seed, n, res), _sources_py(seed, n, res), rtol=1e-6, atol=1e-6)


# ------------------------------------------------------------------ GPU
def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32).ravel()).cuda()


@pytest.mark.gpu
def test_rhs_matches_numpy():
    torch = _torch()
    import fire_sim as F
    res = (32, 64, 32)
    ps = F.Poisson(res, 0.01, "fp32")
    b = torch.empty(res[0] * res[1] * res[2], dtype=torch.float32, device="cuda")
    ps.make_rhs(b, seed=5, n_sources=12, noise=1e-3)
    torch.cuda.synchronize()
    got = b.cpu().numpy().reshape(res[2], res[1], res[0])
    want = _rhs_py(res, 5, 12, 1e-3)
    scale = np.abs(want).max()
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-5 * scale)
    assert abs(float(got.astype(np.float64).mean())) < 1e-6 * scale
    ps.close()


@pytest.mark.gpu
def test_fp32_form_is_the_step_vcycle(oracle_mod):
    """One iteration of the FP32 form is the step's V(2,2) cycle (src/sim.js:588-599) from x = 0."""
    torch = _torch()
    import fire_sim as F
    res, h = (32, 64, 32), 0.01
    rng = np.random.default_rng(4)
    bnp = (FC.smooth_noise((res[2], res[1], res[0]), rng, 2) * 50.0).astype(np.float32)
    ps = F.Poisson(res, h, "fp32")
    b, x = _dev(torch, bnp), torch.zeros(bnp.size, dtype=torch.float32, device="cuda")
    ps.solve(b, x, tol=0.0, max_iters=1)
    r = ps.result()
    assert r["iterations"] == 1
    orc = oracle_mod.OracleSim(res, h)
    orc.put_level(0, "b", bnp)
    orc.put_level(0, "p", np.zeros_like(bnp))
    orc.vcycle()
    want = orc.get_level(0, "p")
    FC.compare(x.cpu().numpy().reshape(want.shape), want, 1e-4, 1e-5, 0, what="fp32 form, one cycle")
    ps.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,res", [("ir32", (64, 128, 64)), ("fp16", (64, 128, 64)), ("bf16", (64, 128, 64)),
                                           ("fp16", (34, 64, 32)), ("bf16", (36, 40, 24))])
def test_solve_to_tolerance(oracle_mod, precision, res):
    """The refinement forms reach 1e-6 relative residual on the solution pair; the FP64 oracle recomputes
    that residual and its CG solution bounds the error.  Grids cover the paired red-black sweep (nx % 4 == 0),
    the single-cell one (34: nx % 4 == 2, odd next level) and a z extent that is no multiple of the residual
    kernel's planes (24)."""
    torch = _torch()
    import fire_sim as F
    h, tol = 0.005, 1e-6
    ps = F.Poisson(res, h, precision)
    n = res[0] * res[1] * res[2]
    b = torch.empty(n, dtype=torch.float32, device="cuda")
    x = torch.zeros(n, dtype=torch.float32, device="cuda")
    lo = torch.zeros(n, dtype=torch.float32, device="cuda")
    ps.make_rhs(b, seed=3, n_sources=32, noise=1e-3)
    ps.solve(b, x, tol=tol, max_iters=40, x_lo=lo)
    r = ps.result()
    assert r["rel_residual"] <= tol and 1 <= r["iterations"] < 40, r
    shape = (res[2], res[1], res[0])
    bnp = b.cpu().numpy().reshape(shape).astype(np.float64)
    x64 = x.cpu().numpy().reshape(shape).astype(np.float64) + lo.cpu().numpy().reshape(shape).astype(np.float64)
    rel64 = np.linalg.norm(bnp - oracle_mod.pressure_apply(x64, h)) / np.linalg.norm(bnp)
    # the device residual is formed in FP32 arithmetic: within a few percent of the FP64 one at 1e-7
    assert rel64 <= 1.05 * tol and rel64 == pytest.approx(r["rel_residual"], rel=0.1), (rel64, r)
    assert ps.residual(b, x, lo) == pytest.approx(r["rel_residual"], rel=1e-6)
    xcg, _, _ = oracle_mod.pressure_cg(bnp, h, tol=1e-12)
    err = np.linalg.norm(x64 - xcg) / np.linalg.norm(xcg)
    assert err < 1e-5, err
    ps.close()


@pytest.mark.gpu
def test_fp32_form_floor(oracle_mod):
    """The step's own cycle iterated on an FP32 x converges to the FP32 representation floor (~1e-5 at this
    size) and no further; the refinement pair goes through it."""
    torch = _torch()
    import fire_sim as F
    res, h = (64, 128, 64), 0.005
    n = res[0] * res[1] * res[2]
    b = torch.empty(n, dtype=torch.float32, device="cuda")
    x = torch.zeros(n, dtype=torch.float32, device="cuda")
    ps = F.Poisson(res, h, "fp32")
    ps.make_rhs(b, seed=3, n_sources=32, noise=1e-3)
    ps.solve(b, x, tol=1e-4, max_iters=40)
    r = ps.result()
    assert r["rel_residual"] <= 1e-4 and r["iterations"] < 40
    shape = (res[2], res[1], res[0])
    rel64 = oracle_mod.pressure_rel_residual(b.cpu().numpy().reshape(shape), x.cpu().numpy().reshape(shape), h)
    assert rel64 == pytest.approx(r["rel_residual"], rel=0.02)
    ps.solve(b, x, tol=0.0, max_iters=30)
    floor = ps.result()["rel_residual"]
    assert 1e-7 < floor < 1e-4
    ps.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_solve_edge_cases(precision):
    torch = _torch()
    import fire_sim as F
    res = (16, 32, 16)
    n = res[0] * res[1] * res[2]
    ps = F.Poisson(res, 0.01, precision)
    b = torch.zeros(n, dtype=torch.float32, device="cuda")
    x = torch.zeros(n, dtype=torch.float32, device="cuda")
    ps.solve(b, x, tol=1e-6, max_iters=10)                    # b = 0: nothing to do
    r = ps.result()
    assert r["iterations"] == 0 and r["rel_residual"] == 0.0 and float(x.abs().max()) == 0.0
    ps.make_rhs(b, seed=1, n_sources=4)
    ps.solve(b, x, tol=0.0, max_iters=3)                      # tol 0: stops at max_iters
    assert ps.result()["iterations"] == 3
    ps.solve(b, x, tol=1e-5, max_iters=30)                    # warm start from the previous x
    r = ps.result()
    assert r["rel_residual"] <= 1e-5 and r["rel_residual_initial"] < 1.0
    with pytest.raises(F.FireError):
        ps.solve(b, b, tol=1e-6)                              # x aliasing b
    with pytest.raises(F.FireError):
        ps.solve(b, x, tol=-1.0)
    with pytest.raises(F.FireError):
        F.Poisson((1, 8, 8), 0.01)
    with pytest.raises(KeyError):
        F.Poisson(res, 0.01, "fp8")
    ps.close()
