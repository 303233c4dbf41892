"""ctypes front-end of the CPU oracle (test infrastructure only).

Two back-ends with one interface:

* ``OracleSolver`` drives ``oracle/liboracle.so``, the plain-C restatement of
  the reference solver (tutorial steps 1-8).  It builds on any host and is the
  parity checker the GPU tests use, and the CPU baseline bench.py times.
* ``RefSolver`` drives ``oracle/_ref/libref<step>.so``: the reference's own
  ``Fluid.cpp`` compiled unmodified (see ``oracle/ref_shim.cpp``).  It exists
  only where the reference checkout was available at build time and is used to
  pin ``OracleSolver`` bit-for-bit.

Only tests, ``__graft_entry__.smoke`` and bench.py's CPU-baseline leg and
its untimed per-field error check may use this module, as the checker.  Bodies are plain tuples
``(type, pos_x, pos_y, scale_x, scale_y, theta, vel_x, vel_y, vel_theta)``
with type 0 = box (full side lengths) and 1 = sphere (diameter in scale_x).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

GS_EULER, GS = 1, 2
PLAIN, SOLID, CURVED, HEAT, VARDENS, FLIP = 3, 4, 5, 6, 7, 8
QD, QT, QU, QV = 0, 1, 2, 3
A_SRC, A_DST, A_PHI, A_VOLUME, A_NORMALX, A_NORMALY = 0, 1, 2, 3, 4, 5
A_R, A_P, A_Z, A_S, A_PRECON, A_ADIAG, A_APLUSX, A_APLUSY, A_UDENS, A_VDENS = range(16, 26)
B_CELL, B_BODY, B_MASK = 0, 1, 2
(PH_FILL_SOLID, PH_HEAT, PH_EXTRAP_T, PH_BUOYANCY, PH_BC, PH_RHS, PH_DENSITIES,
 PH_MATRIX, PH_PRECON, PH_PROJECT, PH_APPLY_P, PH_EXTRAP_DUV, PH_ADVECT,
 PH_P2G, PH_FLIP_COPY, PH_G2P, PH_PADVECT) = range(17)
P_X, P_Y, P_D, P_T, P_U, P_V = range(6)
PCG_CONVERGED, PCG_INITIAL, PCG_CAP = 0, 1, 2


class _Body(C.Structure):
    _fields_ = [("type", C.c_int32), ("pad_", C.c_int32)] + [
        (n, C.c_double) for n in ("pos_x", "pos_y", "scale_x", "scale_y", "theta",
                                  "vel_x", "vel_y", "vel_theta")]


class _Stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("status", C.c_int32), ("max_error", C.c_double)]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "ifl_oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "all", "liboracle.so"],
                       check=True)
    return LIB_PATH


_lib = None


def _oracle_lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        L.ifo_create.restype = vp
        L.ifo_create.argtypes = [i, i, i, d, d, d]
        L.ifo_destroy.argtypes = [vp]
        L.ifo_set_bodies.argtypes = [vp, C.POINTER(_Body), i]
        L.ifo_get_bodies.argtypes = [vp, C.POINTER(_Body)]
        L.ifo_advance_bodies.argtypes = [vp, d]
        L.ifo_add_inflow.argtypes = [vp] + [d] * 8
        L.ifo_update.argtypes = [vp, d]
        L.ifo_phase.argtypes = [vp, i, d]
        L.ifo_set_pinned_iterations.argtypes = [vp, i, i]
        L.ifo_get_stats.argtypes = [vp, C.POINTER(_Stats), C.POINTER(_Stats)]
        L.ifo_array.restype = C.POINTER(C.c_double)
        L.ifo_array.argtypes = [vp, i, i, C.POINTER(i), C.POINTER(i)]
        L.ifo_bytes.restype = C.POINTER(C.c_uint8)
        L.ifo_bytes.argtypes = [vp, i, i, C.POINTER(i), C.POINTER(i)]
        L.ifo_flip.argtypes = [vp, i]
        L.ifo_occupancy.argtypes = [d, d, d, d]
        L.ifo_occupancy.restype = d
        L.ifo_cerp.argtypes = [d, d, d, d, d]
        L.ifo_cerp.restype = d
        L.ifo_to_image.argtypes = [vp, C.c_void_p, i]
        L.ifo_to_image.restype = None
        L.ifo_particles.restype = C.POINTER(C.c_double)
        L.ifo_particles.argtypes = [vp, i, C.POINTER(i)]
        L.ifo_set_particle_count.argtypes = [vp, i]
        L.ifo_flip_init.argtypes = [vp]
        L.ifo_rng_state.restype = C.c_uint32
        L.ifo_rng_state.argtypes = [vp]
        L.ifo_set_rng_state.argtypes = [vp, C.c_uint32]
        L.ifo_frand.restype = C.c_float
        L.ifo_frand.argtypes = [C.POINTER(C.c_uint32)]
        _lib = L
    return _lib


def _view(ptr, w, h, dtype):
    if not ptr:
        return None
    n = w * h
    ctype = C.c_double if dtype == np.float64 else C.c_uint8
    arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n,))
    return arr.reshape(h, w)


def _particle_view(ptr, n):
    if not ptr:
        return None
    return np.ctypeslib.as_array(ptr, shape=(max(n, 0),))[:n]


class OracleSolver:
    """The C restatement of FluidSolver (steps 1-8), FP64, zero-initialised."""

    def __init__(self, variant: int, w: int, h: int, density: float = 0.1,
                 density_soot: float = 1.0, diffusion: float = 0.01):
        self.L = _oracle_lib()
        self.variant, self.w, self.h = variant, w, h
        self.p = self.L.ifo_create(variant, w, h, density, density_soot, diffusion)
        if not self.p:
            raise ValueError("oracle: bad solver parameters")

    def __del__(self):
        if getattr(self, "p", None):
            self.L.ifo_destroy(self.p)
            self.p = None

    def set_bodies(self, bodies):
        arr = (_Body * max(1, len(bodies)))()
        for k, b in enumerate(bodies):
            arr[k].type = int(b[0])
            (arr[k].pos_x, arr[k].pos_y, arr[k].scale_x, arr[k].scale_y, arr[k].theta,
             arr[k].vel_x, arr[k].vel_y, arr[k].vel_theta) = [float(x) for x in b[1:9]]
        if self.L.ifo_set_bodies(self.p, arr, len(bodies)) != 0:
            raise ValueError("oracle: at most 256 bodies")
        self._nb = len(bodies)

    def bodies(self):
        n = getattr(self, "_nb", 0)
        arr = (_Body * max(1, n))()
        self.L.ifo_get_bodies(self.p, arr)
        return [(b.type, b.pos_x, b.pos_y, b.scale_x, b.scale_y, b.theta, b.vel_x, b.vel_y,
                 b.vel_theta) for b in arr[:n]]

    def advance_bodies(self, dt):
        self.L.ifo_advance_bodies(self.p, dt)

    def add_inflow(self, x, y, w, h, d, t, u, v):
        self.L.ifo_add_inflow(self.p, x, y, w, h, d, t, u, v)

    def update(self, dt):
        self.L.ifo_update(self.p, dt)

    def phase(self, ph, dt):
        self.L.ifo_phase(self.p, ph, dt)

    def flip(self, q):
        self.L.ifo_flip(self.p, q)

    def set_pinned_iterations(self, pressure: int, heat: int = -1):
        """-1: stop on the residual test; k >= 0: run exactly k PCG iterations."""
        self.L.ifo_set_pinned_iterations(self.p, pressure, heat)

    def stats(self):
        a, b = _Stats(), _Stats()
        self.L.ifo_get_stats(self.p, C.byref(a), C.byref(b))
        return ((a.iterations, a.status, a.max_error), (b.iterations, b.status, b.max_error))

    def array(self, q: int, which: int):
        w, h = C.c_int(), C.c_int()
        return _view(self.L.ifo_array(self.p, q, which, C.byref(w), C.byref(h)),
                     w.value, h.value, np.float64)

    def bytes(self, q: int, which: int):
        w, h = C.c_int(), C.c_int()
        return _view(self.L.ifo_bytes(self.p, q, which, C.byref(w), C.byref(h)),
                     w.value, h.value, np.uint8)

    def to_image(self, heat: bool = False) -> np.ndarray:
        """FluidSolver::toImage as an (h, w', 4) uint8 array (w' = 2w with heat, steps 6-7)."""
        wide = 2 if (heat and self.variant >= HEAT) else 1
        out = np.zeros((self.h, wide * self.w, 4), dtype=np.uint8)
        self._to_image(out.ctypes.data, 1 if heat else 0)
        return out

    def _to_image(self, ptr, heat):
        self.L.ifo_to_image(self.p, ptr, heat)

    # ---- step 8 particles
    def particle_count(self) -> int:
        n = C.c_int()
        self.L.ifo_particles(self.p, P_X, C.byref(n))
        return n.value

    def particles(self, which: int) -> np.ndarray:
        """Live view of one particle array (P_X .. P_V), length = particle count."""
        n = C.c_int()
        ptr = self.L.ifo_particles(self.p, which, C.byref(n))
        return _particle_view(ptr, n.value)

    def set_particles(self, arrays):
        """Replace the particle state: arrays = (x, y, d, t, u, v), equal lengths."""
        n = len(arrays[0])
        cap = self.w * self.h * 12
        if n > cap:
            raise ValueError("more particles than 12 per cell")
        self.L.ifo_set_particle_count(self.p, n)
        for k, a in enumerate(arrays):
            m = C.c_int()
            ptr = self.L.ifo_particles(self.p, k, C.byref(m))
            np.ctypeslib.as_array(ptr, shape=(cap,))[:n] = np.asarray(a, dtype=np.float64)

    def flip_init(self):
        self.L.ifo_flip_init(self.p)

    @property
    def rng_state(self) -> int:
        return int(self.L.ifo_rng_state(self.p))

    @rng_state.setter
    def rng_state(self, v: int):
        self.L.ifo_set_rng_state(self.p, int(v) & 0xFFFFFFFF)


def frand_stream(state: int, n: int):
    """n values of the reference's frand() from `state`; returns (values, new state)."""
    st = C.c_uint32(state)
    L = _oracle_lib()
    out = np.array([L.ifo_frand(C.byref(st)) for _ in range(n)], dtype=np.float32)
    return out, int(st.value)


def occupancy(d11, d12, d21, d22) -> float:
    return _oracle_lib().ifo_occupancy(d11, d12, d21, d22)


def cerp(a, b, c, d, x) -> float:
    return _oracle_lib().ifo_cerp(a, b, c, d, x)


def ref_available(step: int) -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref{step}.so"))


_ref_libs = {}


def _ref_lib(step):
    if step not in _ref_libs:
        L = C.CDLL(os.path.join(REF_DIR, f"libref{step}.so"))
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        L.ref_create.restype = vp
        L.ref_create.argtypes = [i, i, d, d, d]
        L.ref_destroy.argtypes = [vp]
        L.ref_add_body.argtypes = [vp, i] + [d] * 8
        L.ref_get_body.argtypes = [vp, i, C.POINTER(C.c_double)]
        L.ref_advance_bodies.argtypes = [vp, d]
        L.ref_add_inflow.argtypes = [vp] + [d] * 8
        L.ref_update.argtypes = [vp, d]
        L.ref_pcg_record.argtypes = [i, C.POINTER(i), C.POINTER(i), C.POINTER(d)]
        L.ref_array.restype = C.POINTER(C.c_double)
        L.ref_array.argtypes = [vp, i, i, C.POINTER(i), C.POINTER(i)]
        L.ref_bytes.restype = C.POINTER(C.c_uint8)
        L.ref_bytes.argtypes = [vp, i, i, C.POINTER(i), C.POINTER(i)]
        L.ref_to_image.argtypes = [vp, C.c_void_p, i]
        L.ref_to_image.restype = None
        L.ref_particles.restype = C.POINTER(C.c_double)
        L.ref_particles.argtypes = [vp, i, C.POINTER(i)]
        L.ref_particle_report.restype = i
        L.ref_set_particle_count.argtypes = [vp, i]
        _ref_libs[step] = L
    return _ref_libs[step]


class RefSolver:
    """The reference's own FluidSolver of one tutorial step (zero-initialised)."""

    def __init__(self, variant: int, w: int, h: int, density: float = 0.1,
                 density_soot: float = 1.0, diffusion: float = 0.01):
        self.L = _ref_lib(variant)
        self.variant, self.w, self.h = variant, w, h
        self.p = self.L.ref_create(w, h, density, density_soot, diffusion)
        self._nb = 0
        self.last_records = []

    def __del__(self):
        if getattr(self, "p", None):
            self.L.ref_destroy(self.p)
            self.p = None

    def set_bodies(self, bodies):
        if self._nb:
            raise RuntimeError("reference bodies can only be added once")
        for b in bodies:
            self.L.ref_add_body(self.p, int(b[0]), *[float(x) for x in b[1:9]])
        self._nb = len(bodies)

    def bodies(self):
        out = []
        for k in range(self._nb):
            buf = (C.c_double * 8)()
            self.L.ref_get_body(self.p, k, buf)
            out.append((0,) + tuple(buf))
        return out

    def advance_bodies(self, dt):
        self.L.ref_advance_bodies(self.p, dt)

    def add_inflow(self, x, y, w, h, d, t, u, v):
        self.L.ref_add_inflow(self.p, x, y, w, h, d, t, u, v)

    def update(self, dt):
        n = self.L.ref_update(self.p, dt)
        recs = []
        for k in range(n):
            it, st, e = C.c_int(), C.c_int(), C.c_double()
            self.L.ref_pcg_record(k, C.byref(it), C.byref(st), C.byref(e))
            recs.append((it.value, st.value, e.value))
        self.last_records = recs

    def stats(self):
        """(pressure, heat) records of the last update, as the oracle reports them.
        A solve that returned on its initial residual prints nothing in steps 3-5."""
        recs = list(self.last_records)
        need = 2 if self.variant >= HEAT else 1
        while len(recs) < need:
            recs.append((0, PCG_INITIAL, 0.0))
        if self.variant >= HEAT:
            return recs[1], recs[0]
        return recs[0], (0, PCG_INITIAL, 0.0)

    def array(self, q: int, which: int):
        w, h = C.c_int(), C.c_int()
        return _view(self.L.ref_array(self.p, q, which, C.byref(w), C.byref(h)),
                     w.value, h.value, np.float64)

    def bytes(self, q: int, which: int):
        w, h = C.c_int(), C.c_int()
        return _view(self.L.ref_bytes(self.p, q, which, C.byref(w), C.byref(h)),
                     w.value, h.value, np.uint8)

    def to_image(self, heat: bool = False) -> np.ndarray:
        """FluidSolver::toImage as an (h, w', 4) uint8 array (w' = 2w with heat, steps 6-7)."""
        wide = 2 if (heat and self.variant >= HEAT) else 1
        out = np.zeros((self.h, wide * self.w, 4), dtype=np.uint8)
        self._to_image(out.ctypes.data, 1 if heat else 0)
        return out

    def _to_image(self, ptr, heat):
        self.L.ref_to_image(self.p, ptr, heat)

    # ---- step 8 particles (the reference's frand() stream is one static per
    # process: pin step 8 in a fresh process per reference solver)
    def particle_count(self) -> int:
        n = C.c_int()
        self.L.ref_particles(self.p, P_X, C.byref(n))
        return n.value

    def particles(self, which: int) -> np.ndarray:
        n = C.c_int()
        ptr = self.L.ref_particles(self.p, which, C.byref(n))
        return _particle_view(ptr, n.value)

    def set_particles(self, arrays):
        """Replace the particle state: arrays = (x, y, d, t, u, v), equal lengths."""
        n = len(arrays[0])
        cap = self.w * self.h * 12
        if n > cap:
            raise ValueError("more particles than 12 per cell")
        self.L.ref_set_particle_count(self.p, n)
        for k, a in enumerate(arrays):
            m = C.c_int()
            ptr = self.L.ref_particles(self.p, k, C.byref(m))
            np.ctypeslib.as_array(ptr, shape=(cap,))[:n] = np.asarray(a, dtype=np.float64)


# ------------------------------------------------------ one step from a state
def step_from_state(variant: int, w: int, h: int, state, bodies=(), inflows=(), dt: float = 0.0025,
                    kind: str = "oracle", density: float = 0.1, density_soot: float = 1.0,
                    diffusion: float = 0.01, pinned: int = -1):
    """One FP64 update() from a given state, as the per-step parity checks need it.

    A fresh solver (kind "oracle": the C restatement; "reference": the
    reference's own solver from oracle/_ref) gets `state` — a dict
    {(quantity, A_SRC or A_DST): 2-D array} holding every advected quantity's
    source and target buffers, the whole state that update() carries from one
    step to the next (the pressure starts at zero inside project()) — then the
    bodies (tuples, their state for this step), the inflow rectangles in call
    order and one update(dt).  Returns the pressure, the advected quantities,
    the fluid mask of the pressure grid (solid variants: the reference keeps
    stale pressure at solid cells) and the PCG outcome.  Runs in any process
    (picklable arguments and result), e.g. a spawned pool.
    """
    S = RefSolver if kind == "reference" else OracleSolver
    o = S(variant, w, h, density, density_soot, diffusion)
    if bodies:
        o.set_bodies([tuple(b) for b in bodies])
    for (q, a), arr in state.items():
        o.array(q, a)[...] = np.asarray(arr, dtype=np.float64)
    if pinned >= 0:
        o.set_pinned_iterations(pinned, pinned)
    for r in inflows:
        o.add_inflow(*r)
    o.update(dt)
    qs = [QD, QU, QV] + ([QT] if variant >= HEAT else [])
    out = {q: o.array(q, A_SRC).copy() for q in qs}
    out["p"] = o.array(0, A_P).copy()
    out["fluid"] = (o.bytes(QD, B_CELL) == 0) if variant >= SOLID else np.ones((h, w), dtype=bool)
    out["stats"] = o.stats()
    return out


def field_errors(gpu, ref, variant: int):
    """Max-norm errors of a GPU step against a reference step from the same state.

    p over fluid cells relative to the reference's largest |p| there; u and v
    relative to the largest velocity component (the velocity field's scale);
    d (and T) relative to their own largest value."""
    def rel(a, b, den):
        return float(np.abs(a - b).max() / den) if a.size else 0.0
    m = ref["fluid"]
    pden = max(float(np.abs(ref["p"][m]).max()) if m.any() else 0.0, 1e-300)
    vden = max(float(np.abs(ref[QU]).max()), float(np.abs(ref[QV]).max()), 1e-300)
    out = {"p": rel(gpu["p"][m], ref["p"][m], pden),
           "u": rel(gpu[QU], ref[QU], vden), "v": rel(gpu[QV], ref[QV], vden),
           "d": rel(gpu[QD], ref[QD], max(float(np.abs(ref[QD]).max()), 1e-300))}
    if variant >= HEAT:
        out["T"] = rel(gpu[QT], ref[QT], max(float(np.abs(ref[QT]).max()), 1e-300))
    return out
