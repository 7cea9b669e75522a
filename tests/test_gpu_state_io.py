"""Save and load in the reference's format (save-load.js:91-229) through the
GPUPhysics mirror: a round trip through JSON restores the state exactly
(positions as compensated pairs) and the runs continue identically; a
reference-format file (legacy 'repel' collision name, camera, more particles
than the capacity) loads with its toggles, settings and fields."""
import json

import numpy as np
import pytest

from physsim_gb300 import _native as N
from physsim_gb300.gpu_physics import GeonGPUPhysics

pytestmark = pytest.mark.gpu


class Phys:
    gravityEnabled = True
    coulombEnabled = True
    relativityEnabled = False
    barnesHutEnabled = True
    yukawaEnabled = True
    yukawaMu = 0.2
    bounceFriction = 0.3
    extGravity = 0.05


def backend(cap=64):
    b = GeonGPUPhysics(domainW=100.0, domainH=100.0, maxParticles=cap).init()
    b.setToggles(Phys())
    b.setBoundary(2, 0)                  # loop, torus
    return b


def test_round_trip_is_exact_and_continues_identically(gpu_lib):
    rng = np.random.default_rng(3)
    a = backend()
    for i in range(40):
        a.addParticle({"x": 50 + rng.normal(0, 10), "y": 50 + rng.normal(0, 10), "vx": rng.normal(0, 0.05),
                       "vy": rng.normal(0, 0.05), "mass": rng.lognormal(0, 0.5), "charge": rng.integers(-5, 6) * 0.1,
                       "angw": rng.uniform(-0.2, 0.2), "antimatter": bool(i % 7 == 0)})
    for _ in range(3):
        a.update(1 / 60)
    saved = json.loads(json.dumps(a.serialize()))
    assert saved["version"] == 1 and len(saved["particles"]) == 40
    assert saved["toggles"]["yukawaEnabled"] and not saved["toggles"]["relativityEnabled"]
    assert saved["settings"]["boundary"] == "loop" and saved["settings"]["friction"] == 0.3
    assert sum(p["antimatter"] for p in saved["particles"]) == 6
    b = backend()
    assert b.deserialize(saved)
    again = b.serialize()
    for pa, pb in zip(saved["particles"], again["particles"]):
        for k in ("x", "y", "baseMass", "antimatter"):
            assert pa[k] == pb[k], k
        for k in ("wx", "wy", "mass", "charge", "angw"):
            assert pa[k] == pytest.approx(pb[k], rel=0, abs=0), k
    a.update(1 / 60)
    b.update(1 / 60)
    sa, sb = a.serialize(), b.serialize()
    for pa, pb in zip(sa["particles"], sb["particles"]):
        assert (pa["x"], pa["y"], pa["wx"], pa["wy"]) == (pb["x"], pb["y"], pb["wx"], pb["wy"])
    a.destroy()
    b.destroy()


def test_loads_a_reference_format_file(gpu_lib):
    parts = [{"x": 10.0 + i, "y": 20.0 + 0.5 * i, "wx": 0.01 * i, "wy": -0.02, "mass": 1.0 + 0.1 * i,
              "baseMass": 2.0, "charge": 0.1 * (i % 3 - 1), "angw": 0.0, "antimatter": False} for i in range(80)]
    toggles = {k: False for k, _ in GeonGPUPhysics._SAVE_TOGGLES}
    toggles.update(gravityEnabled=True, coulombEnabled=True, relativityEnabled=True, magneticEnabled=True)
    state = {"version": 1, "particles": parts, "toggles": toggles,
             "settings": {"collision": "repel", "boundary": "bounce", "topology": "klein", "speed": 4, "friction": 0.7},
             "camera": {"x": 0, "y": 0, "zoom": 2}, "yukawaMu": 0.3, "axionMass": 0.05, "hubbleParam": 0.001,
             "higgsMass": 0.5, "extGravity": 0.0, "extGravityAngle": 1.0, "extElectric": 0.2,
             "extElectricAngle": 0.5, "extBz": 0.01}
    b = backend(cap=50)
    with pytest.warns(RuntimeWarning, match="bounce"):
        assert b.deserialize(state)
    assert b.getParticleCount() == 50                       # capacity caps the load (save-load.js:204)
    assert b._collisionMode == N.COL_BOUNCE and b.boundaryMode == 1 and b.topologyMode == 1
    p = b._params()
    assert p.toggles & N.RELATIVITY and p.toggles & N.MAGNETIC and not p.toggles & N.BARNES_HUT
    assert p.bounce_friction == 0.7 and p.yukawa_mu == 0.3 and p.ext_electric == 0.2 and p.ext_bz == 0.01
    st = b._sys.state(f64=True)
    np.testing.assert_array_equal(st["x"], [10.0 + i for i in range(50)])
    w = np.array([0.01 * i for i in range(50)])
    g = np.sqrt(1 + w ** 2 + 0.02 ** 2)
    np.testing.assert_allclose(st["vx"], (w / g).astype(np.float32), rtol=1e-6)   # relativity on: v = w / gamma
    assert b.serialize()["particles"][0]["baseMass"] == 2.0
    assert not b.deserialize({"version": 2})
    b.destroy()
