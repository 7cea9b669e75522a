"""GeonGPUPhysics — the reference's GPUPhysics backend surface over libgeon_cuda.so.

Method names, argument meaning and return conventions follow
src/gpu/gpu-physics.js (constructor :155, addParticle :1857, removeParticle
:1936, setToggles :1969, update :3345, serialize :3749, deserialize :3886,
reset :3973, requestStats/readStats :4146/:4234, getParticleCount :4287,
destroy :4291) so a host that drives GPUPhysics can drive this class.

Differences, all toward the CPU path (src/integrator.js), which is the
authoritative semantics:
  * addParticle takes coordinate velocity (vx, vy) and stores proper
    velocity w = gamma v with |v| clamped below 0.999 (relativity.js:15-25,
    as main.js:504-539 does for the CPU backend); GPUPhysics stores the
    numbers it is given as w directly.
  * removeParticle removes the slot at once and later slots shift down (the
    CPU path's array compaction); ids from getParticleIds() stay stable.
  * Merge collisions run on the device with the CPU path's sequential
    semantics (collisions.js:24-158); the annihilation photons and field
    excitations they would emit are returned as events (collisionEvents)
    instead.  The bounce mode's contact forces are not part of this library.
  * Scalar fields, bosons, heatmap, trails and rendering are not part of
    this library; their GPUPhysics methods are inert stubs.
"""
from __future__ import annotations

import math
import warnings
from typing import Any

import numpy as np

from . import _native as N
from .system import GeonSystem

GPU_MAX_PARTICLES = 512          # src/config.js:128 (the reference's buffer cap)
MAX_SPEED_RATIO = 0.999          # src/config.js:32
BOSON_CHARGE = 0.1               # src/config.js:75
BOUND_NAMES = ["despawn", "bounce", "loop"]
TOPO_NAMES = ["torus", "klein", "rp2"]


def set_velocity(vx: float, vy: float):
    """relativity.js:15-25: clamp |v| < 0.999, return (v, w = gamma v)."""
    speed_sq = vx * vx + vy * vy
    if speed_sq >= 1:
        s = MAX_SPEED_RATIO / math.sqrt(speed_sq)
        vx *= s
        vy *= s
    gamma = 1 / math.sqrt(max(1 - MAX_SPEED_RATIO * MAX_SPEED_RATIO, 1 - vx * vx - vy * vy))
    return (vx, vy), (vx * gamma, vy * gamma)


def quantise_charge(q: float) -> float:
    """main.js:511 / gpu-physics.js:1873: charge is a multiple of 0.1."""
    return round(q / BOSON_CHARGE) * BOSON_CHARGE


def _get(obj: Any, name: str, default=None):
    if isinstance(obj, dict):
        return obj.get(name, default)
    return getattr(obj, name, default)


class GeonGPUPhysics:
    """Drop-in for GPUPhysics; `device` is accepted for signature parity (the CUDA device is the current one)."""

    def __init__(self, device=None, domainW: float = 100.0, domainH: float = 100.0,
                 maxParticles: int = GPU_MAX_PARTICLES):
        self.device = device
        self.domainW = float(domainW)
        self.domainH = float(domainH)
        self.maxParticles = int(maxParticles)
        self.boundaryMode = 0       # despawn
        self.topologyMode = 0       # torus
        self._collisionMode = 0
        self.offX = 0.0
        self.offY = 0.0
        self._toggles = N.GRAVITY | N.COULOMB | N.MAGNETIC | N.GRAVITOMAG | N.ONE_PN | N.RELATIVITY | N.SPIN_ORBIT
        self._flags = N.FLAG_PE | N.FLAG_BREAKDOWN
        self._yukawaMu = 0.15
        self._theta = 0.5
        self._softening = 8.0
        self._ext = dict(ext_gravity=0.0, ext_gravity_angle=math.pi * 0.5, ext_electric=0.0,
                         ext_electric_angle=0.0, ext_bz=0.0)
        self._bounceFriction = 0.4
        self._sys: GeonSystem | None = None
        self._stats = None
        self._selected = -1
        self._ready = False

    # -- lifecycle --------------------------------------------------------------
    def init(self):
        """GPUPhysics.init(): allocates the device buffers."""
        self._sys = GeonSystem(self._params(), self.maxParticles)
        self._ready = True
        return self

    def destroy(self):
        if self._sys:
            self._sys.close()
        self._sys = None
        self._ready = False

    def _params(self) -> N.GeonParams:
        return N.make_params(toggles=self._toggles, flags=self._flags, boundary_mode=self.boundaryMode,
                             topology=self.topologyMode, domain_w=self.domainW, domain_h=self.domainH,
                             off_x=self.offX, off_y=self.offY, theta=self._theta, softening=self._softening,
                             yukawa_mu=self._yukawaMu, bounce_friction=self._bounceFriction,
                             collision_mode=self._library_collision_mode(), **self._ext)

    def _library_collision_mode(self) -> int:
        """Merge runs on the device; bounce (contact forces, integrator.js:669-684)
        is not part of the library: the setting is kept for saving, the run
        proceeds without contact forces and says so."""
        if self._collisionMode == N.COL_BOUNCE:
            warnings.warn("bounce collisions (contact forces) are not simulated by this backend", RuntimeWarning)
            return N.COL_PASS
        return int(self._collisionMode)

    def _sync(self):
        if self._sys:
            self._sys.set_params(self._params())

    # -- toggles (gpu-physics.js:1969-2000) -----------------------------------------
    def setToggles(self, physics):
        bits = [("gravityEnabled", N.GRAVITY), ("coulombEnabled", N.COULOMB), ("magneticEnabled", N.MAGNETIC),
                ("gravitomagEnabled", N.GRAVITOMAG), ("onePNEnabled", N.ONE_PN),
                ("relativityEnabled", N.RELATIVITY), ("spinOrbitEnabled", N.SPIN_ORBIT),
                ("radiationEnabled", N.RADIATION), ("blackHoleEnabled", N.BLACK_HOLE),
                ("yukawaEnabled", N.YUKAWA), ("higgsEnabled", N.HIGGS), ("axionEnabled", N.AXION),
                ("barnesHutEnabled", N.BARNES_HUT)]
        t = 0
        for name, bit in bits:
            if _get(physics, name, False):
                t |= bit
        self._toggles = t
        self._yukawaMu = float(_get(physics, "yukawaMu", self._yukawaMu))
        self._bounceFriction = float(_get(physics, "bounceFriction", self._bounceFriction))
        for key, name in (("ext_gravity", "extGravity"), ("ext_gravity_angle", "extGravityAngle"),
                          ("ext_electric", "extElectric"), ("ext_electric_angle", "extElectricAngle"),
                          ("ext_bz", "extBz")):
            v = _get(physics, name, None)
            if v is not None:
                self._ext[key] = float(v)
        bi = _get(physics, "bosonInterEnabled", None)       # integrator.js:66 (a flag here, not a toggle bit)
        if bi is not None:
            self._flags = (self._flags | N.FLAG_BOSONS) if bi else (self._flags & ~N.FLAG_BOSONS)
        cm = _get(physics, "collisionMode", None)
        if cm is not None:          # COL_* number or the settings string (config.js:10-14)
            self._collisionMode = self.COL_NAMES.index(cm) if cm in self.COL_NAMES else int(cm) if isinstance(cm, int) else 0
        self._sync()

    def setBoundary(self, boundaryMode: int, topologyMode: int = 0):
        self.boundaryMode = int(boundaryMode)
        self.topologyMode = int(topologyMode)
        self._sync()

    def setDomain(self, domainW: float, domainH: float, offX: float = 0.0, offY: float = 0.0):
        self.domainW, self.domainH, self.offX, self.offY = float(domainW), float(domainH), float(offX), float(offY)
        self._sync()

    def setMethod(self, theta: float = 0.5, softening: float = 8.0):
        """theta and softening are run-time parameters here (constants in config.js:44,57)."""
        self._theta, self._softening = float(theta), float(softening)
        self._sync()

    # -- particles -----------------------------------------------------------------------
    @property
    def aliveCount(self) -> int:
        return self._sys.count() if self._sys else 0

    @property
    def simTime(self) -> float:
        return self._sys.sim_time() if self._sys else 0.0

    def getParticleCount(self) -> int:
        return self.aliveCount

    def addParticle(self, p) -> int:
        """{x, y, vx, vy, mass, charge, angw, antimatter} -> slot index, or -1 when full."""
        if self.aliveCount >= self.maxParticles:
            return -1
        m = float(_get(p, "mass", 1.0))
        (_, _), (wx, wy) = set_velocity(float(_get(p, "vx", 0.0)), float(_get(p, "vy", 0.0)))
        q = quantise_charge(float(_get(p, "charge", 0.0)))
        try:
            slot = self._sys.add([_get(p, "x")], [_get(p, "y")], [wx], [wy], [m], [q],
                                 [float(_get(p, "angw", 0.0))], creation_time=self.simTime)
            if _get(p, "antimatter", False):
                self._sys.set_matter(antimatter=[1], first=slot)
            return slot
        except N.GeonError as e:
            if e.code == N.GEON_ERR_FULL:
                return -1
            raise

    def removeParticle(self, idx: int, deathMass: float = 0.0, deathAngVel: float = 0.0):
        if 0 <= idx < self.aliveCount:
            self._sys.remove(idx)

    def patchMass(self, idx: int, newMass: float, newBaseMass: float):
        """Roche-lobe transfer belongs to disintegration, which is not part of this library."""

    def getParticleIds(self) -> np.ndarray:
        return self._sys.ids()

    # -- stepping ---------------------------------------------------------------------------
    def update(self, dt: float):
        """GPUPhysics.update(dt): one frame (gpu-physics.js:3345); returns the substeps taken."""
        if not self._ready or dt <= 0:
            return 0
        return self._sys.update(dt)

    # -- save / load (save format save-load.js:89-120; loading :129-229) ------------------------
    # The toggle names of the saved state (save-load.js:106-111) and their bits.
    _SAVE_TOGGLES = [("gravityEnabled", N.GRAVITY), ("bosonInterEnabled", 0), ("coulombEnabled", N.COULOMB),
                     ("magneticEnabled", N.MAGNETIC), ("gravitomagEnabled", N.GRAVITOMAG),
                     ("relativityEnabled", N.RELATIVITY), ("barnesHutEnabled", N.BARNES_HUT),
                     ("radiationEnabled", N.RADIATION), ("blackHoleEnabled", N.BLACK_HOLE),
                     ("disintegrationEnabled", 0), ("spinOrbitEnabled", N.SPIN_ORBIT), ("onePNEnabled", N.ONE_PN),
                     ("yukawaEnabled", N.YUKAWA), ("axionEnabled", N.AXION), ("expansionEnabled", 0),
                     ("higgsEnabled", N.HIGGS)]
    COL_NAMES = ["pass", "merge", "bounce"]        # COL_PASS, COL_MERGE, COL_BOUNCE (config.js:10-12)

    def serialize(self, sim=None) -> dict:
        """The reference's save state (version 1, save-load.js:91-127): particles
        with position, proper velocity, mass, base mass, charge, angw and the
        antimatter flag; the 16 physics toggles; settings; external fields.
        `sim` (optional) supplies speedScale and camera as the reference reads
        them from the Simulation.  simTime is added (the reference's GPU path
        keeps it on the device)."""
        st = self._sys.state(f64=True)
        n = st["x"].size
        mt = self._sys.matter()
        parts = []
        for i in range(n):
            base, anti = mt["base_mass"][i], mt["antimatter"][i]
            parts.append({"x": float(st["x"][i]), "y": float(st["y"][i]), "wx": float(st["wx"][i]),
                          "wy": float(st["wy"][i]), "mass": float(st["mass"][i]), "baseMass": float(base),
                          "charge": float(st["charge"][i]), "angw": float(st["angw"][i]), "antimatter": bool(anti)})
        toggles = {name: bool(bit and (self._toggles & bit)) for name, bit in self._SAVE_TOGGLES}
        toggles["bosonInterEnabled"] = bool(self._flags & N.FLAG_BOSONS)
        settings = {"collision": self.COL_NAMES[int(self._collisionMode) % 3] if isinstance(self._collisionMode, int)
                    else str(self._collisionMode),
                    "boundary": BOUND_NAMES[self.boundaryMode], "topology": TOPO_NAMES[self.topologyMode],
                    "speed": float(_get(sim, "speedScale", 1.0)) if sim is not None else 1.0,
                    "friction": self._bounceFriction}
        state = {"version": 1, "particles": parts, "toggles": toggles, "settings": settings,
                 "yukawaMu": self._yukawaMu, "axionMass": None, "hubbleParam": None, "higgsMass": None,
                 "extGravity": self._ext["ext_gravity"], "extGravityAngle": self._ext["ext_gravity_angle"],
                 "extElectric": self._ext["ext_electric"], "extElectricAngle": self._ext["ext_electric_angle"],
                 "extBz": self._ext["ext_bz"], "simTime": self.simTime}
        cam = _get(sim, "camera", None) if sim is not None else None
        if cam is not None:
            state["camera"] = {"x": _get(cam, "x", 0.0), "y": _get(cam, "y", 0.0), "zoom": _get(cam, "zoom", 1.0)}
        return state

    def deserialize(self, state: dict, sim=None) -> bool:
        """loadState (save-load.js:129-229): restores toggles, external fields,
        friction and the boundary / topology / collision settings, then the
        particles (at most maxParticles; loaded particles always existed,
        :212; coordinate velocity from w as :220-223 derive it)."""
        if not state or state.get("version") != 1:
            return False
        tg = state.get("toggles") or {}
        if tg:
            t = 0
            for name, bit in self._SAVE_TOGGLES:
                if bit and tg.get(name, False):
                    t |= bit
            self._toggles = t
            if tg.get("bosonInterEnabled", False):
                self._flags |= N.FLAG_BOSONS
            else:
                self._flags &= ~N.FLAG_BOSONS
        for key, name in (("ext_gravity", "extGravity"), ("ext_gravity_angle", "extGravityAngle"),
                          ("ext_electric", "extElectric"), ("ext_electric_angle", "extElectricAngle"),
                          ("ext_bz", "extBz")):
            if state.get(name) is not None:
                self._ext[key] = float(state[name])
        if state.get("yukawaMu") is not None:
            self._yukawaMu = float(state["yukawaMu"])
        st = state.get("settings") or {}
        if st.get("friction") is not None:
            self._bounceFriction = float(st["friction"])
        if st.get("boundary") in BOUND_NAMES:
            self.boundaryMode = BOUND_NAMES.index(st["boundary"])
        if st.get("topology") in TOPO_NAMES:
            self.topologyMode = TOPO_NAMES.index(st["topology"])
        col = "bounce" if st.get("collision") == "repel" else st.get("collision", "pass")   # save-load.js:183-184
        if col in self.COL_NAMES:
            self._collisionMode = self.COL_NAMES.index(col)
        self._sync()
        parts = (state.get("particles") or [])[: self.maxParticles]
        f = lambda k, d=0.0: np.array([float(pp.get(k, d) if pp.get(k, d) is not None else d) for pp in parts])
        self._sys.upload_f64(f("x"), f("y"), f("wx"), f("wy"), f("mass", 1.0), f("charge"), f("angw"),
                             sim_time=float(state.get("simTime", 0.0) or 0.0))
        if parts:
            self._sys.set_matter(antimatter=np.array([1 if pp.get("antimatter", False) else 0 for pp in parts]),
                                 base_mass=f("baseMass", 0.0) + np.where([pp.get("baseMass") is None for pp in parts],
                                                                      f("mass", 1.0), 0.0))
        return True

    def reset(self):
        self._sys.reset()
        self._stats = None

    def setBosonPool(self, photons=(), pions=(), leptons=()):
        """The Simulation's alive bosons for the boson tree (integrator.js:263-277):
        objects with pos {x, y} (or x, y), _srcMass and, for pions and
        leptons, charge and vSq.  With bosonInterEnabled, every force pass of
        update() adds their gravity on the particles (forces.js:788-804)."""
        rows = []
        for kind, group in ((0, photons), (1, pions), (1, leptons)):
            for b in group:
                if not _get(b, "alive", True):
                    continue
                pos = _get(b, "pos", None)
                x = float(_get(pos, "x") if pos is not None else _get(b, "x"))
                y = float(_get(pos, "y") if pos is not None else _get(b, "y"))
                q = 0.0 if kind == 0 else float(_get(b, "charge", 0.0))
                rows.append((x, y, float(_get(b, "_srcMass", 0.0)), q, kind,
                             0.0 if kind == 0 else float(_get(b, "vSq", 0.0))))
        self._sys.set_bosons(np.array(rows, dtype=np.float64).reshape(-1, 6))

    def bosonKicks(self, dt: float) -> np.ndarray:
        """Kicks of the pool on itself, in setBosonPool order (photons, pions,
        leptons): gravity (forces.js:812-856, before the photons' speed
        renormalisation) plus, with Coulomb on, Coulomb between pions and
        leptons (forces.js:878-901).  Photons add the kick to their velocity,
        pions and leptons to w."""
        what = (1 if self._toggles & N.GRAVITY else 0) | (2 if self._toggles & N.COULOMB else 0)
        return self._sys.boson_kicks(dt, what)

    def collisionEvents(self) -> np.ndarray:
        """Events of the last update (rows type, x, y, energy, px, py; type 1
        annihilation, 2 merge): what handleCollisions returns to the caller
        for photon bursts and field excitations (integrator.js:1383-1414)."""
        return self._sys.collision_events()

    # -- stats (gpu-physics.js:4146-4283) ----------------------------------------------------
    def requestStats(self, selectedGpuIdx: int = -1):
        self._selected = int(selectedGpuIdx)
        self._stats = self._sys.stats()

    def readStats(self):
        if self._stats is None:
            return None
        s = self._stats
        self._stats = None
        res = {"linearKE": s["linear_ke"], "spinKE": s["spin_ke"], "px": s["px"], "py": s["py"],
               "orbitalAngMom": s["orbital_ang_mom"], "spinAngMom": s["spin_ang_mom"], "comX": s["com_x"],
               "comY": s["com_y"], "totalMass": s["total_mass"], "aliveCount": s["alive_count"], "pe": s["pe"],
               "selected": None}
        i = self._selected
        if 0 <= i < s["alive_count"]:
            st = self._sys.state()
            f = self._sys.forces()
            res["selected"] = {
                "posX": st["x"][i], "posY": st["y"][i], "velWX": st["wx"][i], "velWY": st["wy"][i],
                "mass": st["mass"][i], "charge": st["charge"][i], "angW": st["angw"][i],
                "velX": st["vx"][i], "velY": st["vy"][i], "angVel": st["angVel"][i],
                "forceGravity": {"x": f["grav_x"][i], "y": f["grav_y"][i]},
                "forceCoulomb": {"x": f["coul_x"][i], "y": f["coul_y"][i]},
                "forceMagnetic": {"x": f["mag_x"][i], "y": f["mag_y"][i]},
                "forceGravitomag": {"x": f["gm_x"][i], "y": f["gm_y"][i]},
                "force1PN": {"x": f["f1pn_x"][i], "y": f["f1pn_y"][i]},
                "forceYukawa": {"x": f["yuk_x"][i], "y": f["yuk_y"][i]},
                "forceExternal": {"x": f["ext_x"][i], "y": f["ext_y"][i]},
            }
        return res

    # -- inert stubs for the out-of-scope parts of GPUPhysics --------------------------------
    def _stub(self, *a, **k):
        return None

    setHeatmapEnabled = setTrailsEnabled = dispatchHeatmap = resetFields = _stub
    hitTest = _stub

    def getFieldData(self, *a, **k):
        return np.zeros(0, dtype=np.float32)
