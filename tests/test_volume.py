"""Volume rendering of the fire (src/renderer.js pLights / pVolume, src/blackbody.js): the blackbody LUT
against a Python restatement, and the CUDA lights and ray march against the CPU restatement on a burning
fire."""
import math

import numpy as np
import pytest

import fire_cases as FC

H, C, KB = 6.62607015e-34, 2.99792458e8, 1.380649e-23


def _cie(l):
    g = lambda x, mu, s1, s2: math.exp(-0.5 * ((x - mu) / (s1 if x < mu else s2)) ** 2)
    return (1.056 * g(l, 599.8, 37.9, 31.0) + 0.362 * g(l, 442.0, 16.0, 26.7) - 0.065 * g(l, 501.1, 20.4, 26.2),
            0.821 * g(l, 568.8, 46.9, 40.5) + 0.286 * g(l, 530.9, 16.3, 31.1),
            1.217 * g(l, 437.0, 11.8, 36.0) + 0.681 * g(l, 459.0, 26.0, 13.8))


def _bb_xyz(T, soot=False):
    X = Y = Z = 0.0
    for l in range(380, 781, 2):
        p = (2 * H * C * C) / ((l * 1e-9) ** 5 * (math.exp((H * C) / (l * 1e-9 * KB * T)) - 1)) * ((l / 550) ** -1.39 if soot else 1)
        x, y, z = _cie(l)
        X, Y, Z = X + p * x, Y + p * y, Z + p * z
    return np.array([X, Y, Z])


def _lut_py(n=64, tmin=400.0, tmax=3000.0, twb=5000.0):
    XYZ2RGB = np.array([[3.2404542, -1.5371385, -0.4985314], [-0.9692660, 1.8760108, 0.0415560], [0.0556434, -0.2040259, 1.0572252]])
    XYZ2LMS = np.array([[0.8951, 0.2664, -0.1614], [-0.7502, 1.7135, 0.0367], [0.0389, -0.0685, 1.0296]])
    w = _bb_xyz(twb)
    src, dst = XYZ2LMS @ (w / w[1]), XYZ2LMS @ np.array([0.95047, 1.0, 1.08883])
    conv = XYZ2RGB @ np.linalg.inv(XYZ2LMS) @ np.diag(dst / src) @ XYZ2LMS
    ref = _bb_xyz(1500)[1]
    out = np.zeros((2, n, 4))
    for row in range(2):
        for i in range(n):
            xyz = _bb_xyz(tmin + (tmax - tmin) * i / (n - 1), row == 1) / ref
            out[row, i, :3] = np.maximum(0, conv @ xyz)
            out[row, i, 3] = xyz[1]
    return out


def test_blackbody_lut_matches_python():
    import fire_sim as F
    got = F.blackbody_lut(64, 400.0, 3000.0, 5000.0)
    want = _lut_py(64)
    np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-12)
    # a 1500 K blackbody has unit luminance in the LUT's units, and soot is bluer than a blackbody
    temps = 400 + 2600 * np.arange(64) / 63
    assert np.interp(1500, temps, np.log(got[0, :, 3])) == pytest.approx(0.0, abs=0.02)
    assert got[1, 40, 2] / got[1, 40, 0] > got[0, 40, 2] / got[0, 40, 0]


# ------------------------------------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def campfire():
    import fire_sim as F
    return F.build_campfire(7)


@pytest.mark.gpu
def test_volume_matches_oracle(oracle_mod, campfire):
    import fire_sim as F
    dt = FC.C1["dt"]
    sim = F.FireSim(res=FC.C1["res"], size=FC.C1["size"], logs=campfire, vcycles=4)
    sim.step(dt, 90)
    sim.sync()
    vol = F.Volume(sim, width=128, height=192, vol_scale=0.5)
    assert (vol.vw, vol.vh) == (64, 96)
    vol.set_camera((0.35, 0.45, 1.3), (0.0, 0.42, 0.0), 40.0, jitter=(0.3, -0.2))
    vol.set_params({"smokeScat": 0.05, "sootScat": 0.03})
    S, S2 = sim.download("S"), sim.download("S2")
    curl = sim.download("curl").astype(np.float32)
    lut = F.blackbody_lut(1024, 400.0, 3000.0, 5000.0).reshape(-1, 4)
    lstate = np.zeros((24, 4), np.float32)
    for k, (time, frame) in enumerate(((0.75, 3), (0.75 + dt, 4))):   # a filter reset, then a filtered render
        U = vol.uniforms(time, frame)
        assert (U[53] < 0) == (k == 0)                                    # lightDt
        vol.render(time, frame)
        lights = vol.lights()
        want_l, lstate = oracle_mod.volume_lights(U, S, lut, lstate)
        np.testing.assert_allclose(lights, want_l, rtol=1e-4, atol=1e-6 * np.abs(want_l).max())
        img = vol.image()
        want, aux = oracle_mod.volume_render(U, S, S2, curl, lut, lights)
        scale = float(np.abs(want[..., :3]).max())
        assert scale > 0 and (want[..., 3] < 0.99).any()                 # the fire is in view and absorbs
        bad = np.abs(img - want) > 1e-3 * np.abs(want) + 1e-4 * max(scale, 1.0)
        assert bad.mean() < 0.005, (k, bad.mean(), float(np.abs(img - want).max()))
        np.testing.assert_allclose(vol.aux()[..., 0], aux[..., 0], rtol=1e-3, atol=1e-6)
    vol.close()
    sim.close()
