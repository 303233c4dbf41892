"""Python mirror of the reference FluidSolver surface over the GB300 C ABI.

The classes here follow the reference's own interface (tunabrain/
incremental-fluids): ``FluidSolver(w, h, density)`` (step 3),
``FluidSolver(w, h, density, bodies)`` (steps 4/5),
``FluidSolver(w, h, rhoAir, rhoSoot, diffusion, bodies)`` (steps 6/7),
``addInflow``, ``update``, ``ambientT``, and ``SolidBox`` / ``SolidSphere``
bodies with ``update(dt)``.  Field readback (``read_field``) replaces the
reference's PNG output.  Every call goes through ``libifluids.so``
(``include/ifluids.h``); there is no CPU fallback: if the library is missing
or no GPU is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Iterable, List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libifluids.so")

# include/ifluids.h constants
OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT, ERR_UNSUPPORTED = 0, -1, -2, -3, -4, -5
GS_EULER, GS = 1, 2
PLAIN, SOLID, CURVED, HEAT, VARDENS, FLIP = 3, 4, 5, 6, 7, 8
FP64, FP32 = 0, 1
DT_F64, DT_F32, DT_U8 = 0, 1, 2
Q_D, Q_T, Q_U, Q_V = 0, 1, 2, 3
A_SRC, A_DST, A_PHI, A_VOLUME, A_NORMALX, A_NORMALY, A_CELL, A_BODY = 0, 1, 2, 3, 4, 5, 8, 9
F_R, F_P, F_Z, F_S, F_PRECON, F_ADIAG, F_APLUSX, F_APLUSY, F_UDENS, F_VDENS = range(16, 26)
(PH_FILL_SOLID, PH_HEAT, PH_EXTRAP_T, PH_BUOYANCY, PH_BC, PH_RHS, PH_DENSITIES, PH_MATRIX,
 PH_PRECON, PH_PROJECT, PH_APPLY_P, PH_EXTRAP_DUV, PH_ADVECT,
 PH_P2G, PH_FLIP_COPY, PH_G2P, PH_PADVECT) = range(17)
P_X, P_Y, P_D, P_T, P_U, P_V = range(6)
CELL_FLUID, CELL_SOLID, CELL_EMPTY = 0, 1, 2
PCG_CONVERGED, PCG_INITIAL, PCG_CAP = 0, 1, 2

EXPORTS = ("ifl_default_params", "ifl_create", "ifl_destroy", "ifl_set_bodies", "ifl_get_bodies",
           "ifl_advance_bodies", "ifl_add_inflow", "ifl_update", "ifl_run_phase", "ifl_ambient_t",
           "ifl_field_shape", "ifl_read_field", "ifl_write_field", "ifl_render", "ifl_flip", "ifl_get_stats",
           "ifl_flip_init", "ifl_particle_count", "ifl_read_particles", "ifl_write_particles",
           "ifl_set_particle_count", "ifl_get_rng_state", "ifl_set_rng_state",
           "ifl_set_pinned_iterations", "ifl_set_wait_limit", "ifl_synchronize", "ifl_stream", "ifl_launch_count",
           "ifl_set_timing", "ifl_get_timing", "ifl_pcg_solve_noalloc",
           "ifl_batch_default_options", "ifl_batch_create", "ifl_batch_destroy", "ifl_batch_set_inflows",
           "ifl_batch_update", "ifl_batch_get_stats", "ifl_batch_get_info", "ifl_batch_stream",
           "ifl_batch_last_error", "ifl_batch_plan_teams", "ifl_server_default_params", "ifl_server_create",
           "ifl_server_destroy", "ifl_server_now", "ifl_server_submit", "ifl_server_step",
           "ifl_server_completions", "ifl_server_field_shape", "ifl_server_read_field", "ifl_server_request_stats", "ifl_server_release",
           "ifl_server_get_info", "ifl_server_last_error", "ifl_device_bytes", "ifl_last_error", "ifl_version")


def field_id(quantity: int, array: int) -> int:
    return (quantity << 8) | array


_NAMED = {"d": field_id(Q_D, A_SRC), "t": field_id(Q_T, A_SRC), "u": field_id(Q_U, A_SRC),
          "v": field_id(Q_V, A_SRC), "p": F_P, "r": F_R, "z": F_Z, "s": F_S, "precon": F_PRECON,
          "adiag": F_ADIAG, "aplusx": F_APLUSX, "aplusy": F_APLUSY, "udens": F_UDENS, "vdens": F_VDENS}


class Params(C.Structure):
    _fields_ = [("variant", C.c_int32), ("w", C.c_int32), ("h", C.c_int32), ("precision", C.c_int32),
                ("density_air", C.c_double), ("density_soot", C.c_double), ("diffusion", C.c_double),
                ("max_iter_pressure", C.c_int32), ("max_iter_heat", C.c_int32), ("stream", C.c_void_p),
                ("device", C.c_int32), ("pad_", C.c_int32)]


K_PCG, K_ASSEMBLE, K_ADVECT, K_SOLID, K_EXTRAPOLATE, K_FACES = range(6)
K_NAMES = ("pcg", "assemble", "advect", "solid", "extrapolate", "faces", "particles")


class Timing(C.Structure):
    _fields_ = [("ms", C.c_double * 7), ("launches", C.c_int64 * 7), ("pcg_iterations", C.c_int64)]


class _CBody(C.Structure):
    _fields_ = [("type", C.c_int32), ("pad_", C.c_int32)] + [
        (n, C.c_double) for n in ("pos_x", "pos_y", "scale_x", "scale_y", "theta", "vel_x", "vel_y",
                                  "vel_theta")]


class PcgStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("status", C.c_int32), ("max_error", C.c_double)]


class StepStats(C.Structure):
    _fields_ = [("pressure", PcgStats), ("heat", PcgStats), ("device_flags", C.c_uint32),
                ("steps", C.c_uint32)]


class Inflow(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x", "y", "w", "h", "d", "t", "u", "v")]


class BatchOptions(C.Structure):
    _fields_ = [("threads", C.c_int32), ("strips_per_block", C.c_int32), ("stages", C.c_int32),
                ("use_graph", C.c_int32), ("tune_iterations", C.c_int32), ("max_team_blocks", C.c_int32),
                ("tile_tune", C.c_int32), ("pad_", C.c_int32), ("tile_w", C.c_int32 * 8), ("tile_h", C.c_int32 * 8)]


# Tiled phases of a batch step (ifl_batch_options.tile_w / tile_h, ifl_batch_info)
TILE_PHASES = ("fill", "bc", "assemble", "heat_assemble", "advect", "apply", "buoyancy", "mask")
TILE_SHAPES = ((32, 8), (32, 4), (64, 4), (16, 16), (128, 2), (64, 2))


class BatchInfo(C.Structure):
    _fields_ = [("members", C.c_int32), ("threads", C.c_int32), ("strips_per_block", C.c_int32),
                ("stages", C.c_int32), ("grid", C.c_int32), ("graph", C.c_int32), ("candidates", C.c_int32),
                ("pad_", C.c_int32), ("candidate_ms", C.c_double * 8), ("last_step_ms", C.c_double),
                ("last_pcg_ms", C.c_double), ("launches", C.c_int64), ("steps", C.c_int64),
                ("h2d_bytes_last_step", C.c_int64), ("d2h_bytes_last_step", C.c_int64),
                ("tile_w", C.c_int32 * 8), ("tile_h", C.c_int32 * 8), ("tile_ms", C.c_double * 8)]


class ServerParams(C.Structure):
    _fields_ = [("variant", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32), ("max_active", C.c_int32),
                ("dt", C.c_double), ("hbm_budget_bytes", C.c_int64), ("dry_run", C.c_int32), ("pad_", C.c_int32),
                ("batch", BatchOptions)]


class Request(C.Structure):
    _fields_ = [("w", C.c_int32), ("h", C.c_int32), ("steps", C.c_int32), ("n_bodies", C.c_int32),
                ("n_inflows", C.c_int32), ("pad_", C.c_int32), ("bodies", C.c_void_p), ("inflows", C.c_void_p),
                ("arrival", C.c_double)]


class Completion(C.Structure):
    _fields_ = [("id", C.c_int64), ("w", C.c_int32), ("h", C.c_int32), ("steps", C.c_int32), ("pad_", C.c_int32),
                ("arrival", C.c_double), ("admitted", C.c_double), ("finished", C.c_double),
                ("device_bytes", C.c_int64)]


class ServerInfo(C.Structure):
    _fields_ = [("active", C.c_int32), ("queued", C.c_int32), ("bytes_in_use", C.c_int64),
                ("cell_steps", C.c_int64), ("steps", C.c_int64), ("rebuilds", C.c_int64), ("threads", C.c_int32),
                ("strips_per_block", C.c_int32), ("stages", C.c_int32), ("pad_", C.c_int32),
                ("peak_queued", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("rebuild_ms", C.c_double)]


class IflError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ifluids error {code}: {msg}")
        self.code = code


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libifluids.so and declare its C signatures (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"libifluids.so not built ({path}); run incremental-fluids_gb300/build.py")
    L = C.CDLL(path)
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    L.ifl_default_params.argtypes = [C.POINTER(Params), i, i, i]
    L.ifl_default_params.restype = None
    L.ifl_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.ifl_destroy.argtypes = [vp]
    L.ifl_set_bodies.argtypes = [vp, C.POINTER(_CBody), i]
    L.ifl_get_bodies.argtypes = [vp, C.POINTER(_CBody), i, C.POINTER(i)]
    L.ifl_advance_bodies.argtypes = [vp, d]
    L.ifl_add_inflow.argtypes = [vp] + [d] * 8
    L.ifl_update.argtypes = [vp, d]
    L.ifl_run_phase.argtypes = [vp, i, d]
    L.ifl_ambient_t.argtypes = [vp]
    L.ifl_ambient_t.restype = d
    L.ifl_field_shape.argtypes = [vp, i, C.POINTER(i), C.POINTER(i)]
    L.ifl_read_field.argtypes = [vp, i, vp, sz, i]
    L.ifl_write_field.argtypes = [vp, i, vp, sz, i]
    L.ifl_flip.argtypes = [vp, i]
    L.ifl_flip_init.argtypes = [vp]
    L.ifl_particle_count.argtypes = [vp, C.POINTER(i)]
    L.ifl_read_particles.argtypes = [vp, i, vp, i, C.POINTER(i)]
    L.ifl_write_particles.argtypes = [vp, i, vp, i]
    L.ifl_set_particle_count.argtypes = [vp, i]
    L.ifl_get_rng_state.argtypes = [vp, C.POINTER(C.c_uint32)]
    L.ifl_set_rng_state.argtypes = [vp, C.c_uint32]
    L.ifl_render.argtypes = [vp, i, vp, sz, i]
    L.ifl_get_stats.argtypes = [vp, C.POINTER(StepStats)]
    L.ifl_set_pinned_iterations.argtypes = [vp, i, i]
    L.ifl_set_wait_limit.argtypes = [vp, C.c_int64]
    L.ifl_synchronize.argtypes = [vp]
    L.ifl_set_timing.argtypes = [vp, i]
    L.ifl_pcg_solve_noalloc.argtypes = [i, i, vp, vp, vp, vp, vp, i, vp, vp]
    L.ifl_get_timing.argtypes = [vp, C.POINTER(Timing)]
    L.ifl_stream.argtypes = [vp]
    L.ifl_stream.restype = vp
    L.ifl_launch_count.argtypes = [vp]
    L.ifl_launch_count.restype = C.c_int64
    L.ifl_last_error.argtypes = [vp]
    L.ifl_last_error.restype = C.c_char_p
    L.ifl_version.restype = C.c_char_p
    L.ifl_batch_default_options.argtypes = [C.POINTER(BatchOptions)]
    L.ifl_batch_default_options.restype = None
    L.ifl_batch_create.argtypes = [C.POINTER(vp), i, C.POINTER(BatchOptions), C.POINTER(vp)]
    L.ifl_batch_destroy.argtypes = [vp]
    L.ifl_batch_set_inflows.argtypes = [vp, i, C.POINTER(Inflow), i]
    L.ifl_batch_update.argtypes = [vp, d]
    L.ifl_batch_get_stats.argtypes = [vp, C.POINTER(StepStats), i]
    L.ifl_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
    L.ifl_batch_stream.argtypes = [vp]
    L.ifl_batch_stream.restype = vp
    L.ifl_batch_last_error.argtypes = [vp]
    L.ifl_batch_last_error.restype = C.c_char_p
    L.ifl_batch_plan_teams.argtypes = [i, i, i, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int)]
    L.ifl_server_default_params.argtypes = [C.POINTER(ServerParams), i, i]
    L.ifl_server_default_params.restype = None
    L.ifl_server_create.argtypes = [C.POINTER(ServerParams), C.POINTER(vp)]
    L.ifl_server_destroy.argtypes = [vp]
    L.ifl_server_now.argtypes = [vp]
    L.ifl_server_now.restype = d
    L.ifl_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_int64)]
    L.ifl_server_step.argtypes = [vp, C.POINTER(i), C.POINTER(i)]
    L.ifl_server_completions.argtypes = [vp, C.POINTER(Completion), i, C.POINTER(i)]
    L.ifl_server_read_field.argtypes = [vp, C.c_int64, i, vp, sz, i]
    L.ifl_server_field_shape.argtypes = [vp, C.c_int64, i, C.POINTER(i), C.POINTER(i)]
    L.ifl_server_request_stats.argtypes = [vp, C.c_int64, C.POINTER(StepStats)]
    L.ifl_server_release.argtypes = [vp, C.c_int64]
    L.ifl_server_get_info.argtypes = [vp, C.POINTER(ServerInfo)]
    L.ifl_server_last_error.argtypes = [vp]
    L.ifl_server_last_error.restype = C.c_char_p
    L.ifl_device_bytes.argtypes = [C.POINTER(Params)]
    L.ifl_device_bytes.restype = C.c_int64
    _lib = L
    return L


def pcg_solve_noalloc(w: int, h: int, adiag: int, aplusx: int, aplusy: int, rhs: int, p: int,
                      max_iter: int, stats: int, stream: int = 0) -> int:
    """ifl_pcg_solve_noalloc on device pointers (see include/ifluids.h); returns the status."""
    return int(load_library().ifl_pcg_solve_noalloc(w, h, adiag, aplusx, aplusy, rhs, p, max_iter, stats,
                                                    stream or None))


class SolidBody:
    """Rigid body of the reference (4-solid-boundaries/Fluid.cpp:79-149)."""

    type = 0

    def __init__(self, pos_x, pos_y, scale_x, scale_y, theta, vel_x, vel_y, vel_theta):
        self.pos_x, self.pos_y = float(pos_x), float(pos_y)
        self.scale_x, self.scale_y = float(scale_x), float(scale_y)
        self.theta = float(theta)
        self.vel_x, self.vel_y, self.vel_theta = float(vel_x), float(vel_y), float(vel_theta)

    def update(self, timestep: float):
        """SolidBody::update: explicit Euler step of position and angle."""
        self.pos_x += self.vel_x * timestep
        self.pos_y += self.vel_y * timestep
        self.theta += self.vel_theta * timestep

    def as_tuple(self):
        return (self.type, self.pos_x, self.pos_y, self.scale_x, self.scale_y, self.theta,
                self.vel_x, self.vel_y, self.vel_theta)


class SolidBox(SolidBody):
    """SolidBox(x, y, sx, sy, t, vx, vy, vt): full side lengths sx, sy."""
    type = 0


class SolidSphere(SolidBody):
    """SolidSphere(x, y, s, t, vx, vy, vt): diameter s."""
    type = 1

    def __init__(self, pos_x, pos_y, scale, theta, vel_x, vel_y, vel_theta):
        super().__init__(pos_x, pos_y, scale, scale, theta, vel_x, vel_y, vel_theta)


def _body_tuple(b):
    return b.as_tuple() if isinstance(b, SolidBody) else tuple(b)


class FluidSolver:
    """Device-resident FluidSolver.

    Positional forms follow the reference constructors::

        FluidSolver(w, h, density)                          # 3-conjugate-gradients (variant=1:
                                                            #   1-matrixless, 2: 2-better-advection)
        FluidSolver(w, h, density, bodies)                  # 4-solid-boundaries (variant=5: curved)
        FluidSolver(w, h, rhoAir, rhoSoot, diffusion, bodies)  # 7-variable-density (variant=6: heat,
                                                               #   variant=8: 8-flip, FP64 only)

    Bodies are held by reference as in the reference: before every update()
    their current state is sent to the device, so callers move them with
    ``SolidBody.update(dt)`` between steps exactly as the reference's main()
    does.  ``precision`` selects the FP64 drop-in or the FP32 form.
    """

    def __init__(self, w: int, h: int, *args, variant: Optional[int] = None, precision: int = FP64,
                 max_iter_pressure: Optional[int] = None, max_iter_heat: Optional[int] = None,
                 stream: Optional[int] = None, device: int = 0):
        self._L = load_library()
        bodies: Sequence = ()
        soot = diffusion = None
        if len(args) == 1:
            density = args[0]
            v = PLAIN
        elif len(args) == 2:
            density, bodies = args
            v = SOLID
        elif len(args) == 4:
            density, soot, diffusion, bodies = args
            v = VARDENS
        else:
            raise TypeError("FluidSolver(w, h, density[, bodies]) or (w, h, rhoAir, rhoSoot, diffusion, bodies)")
        if variant is not None:
            v = variant
        p = Params()
        self._L.ifl_default_params(C.byref(p), v, int(w), int(h))
        p.precision = precision
        p.density_air = float(density)
        if soot is not None:
            p.density_soot = float(soot)
        if diffusion is not None:
            p.diffusion = float(diffusion)
        if max_iter_pressure is not None:
            p.max_iter_pressure = int(max_iter_pressure)
        if max_iter_heat is not None:
            p.max_iter_heat = int(max_iter_heat)
        p.stream = stream
        p.device = int(device)
        h_ = C.c_void_p()
        rc = self._L.ifl_create(C.byref(p), C.byref(h_))
        if rc != OK:
            raise IflError(rc, "ifl_create failed (is a GPU present and the size valid?)")
        self._h = h_
        self.variant, self.w, self.h, self.precision = v, int(w), int(h), precision
        self._bodies: List = list(bodies)
        self._uploaded = None

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._L.ifl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != OK:
            msg = self._L.ifl_last_error(self._h)
            raise IflError(rc, f"{what}: {msg.decode() if msg else ''}")

    # -- bodies
    @property
    def bodies(self):
        return self._bodies

    def set_bodies(self, bodies: Iterable):
        self._bodies = list(bodies)
        self._uploaded = None

    def _sync_bodies(self):
        if self.variant < SOLID:
            return
        cur = tuple(_body_tuple(b) for b in self._bodies)
        if cur == self._uploaded:
            return
        arr = (_CBody * max(1, len(cur)))()
        for k, b in enumerate(cur):
            arr[k].type = int(b[0])
            (arr[k].pos_x, arr[k].pos_y, arr[k].scale_x, arr[k].scale_y, arr[k].theta, arr[k].vel_x,
             arr[k].vel_y, arr[k].vel_theta) = [float(x) for x in b[1:9]]
        self._check(self._L.ifl_set_bodies(self._h, arr, len(cur)), "set_bodies")
        self._uploaded = cur

    # -- reference surface
    def addInflow(self, x, y, w, h, d, *rest):
        """addInflow(x, y, w, h, d, u, v) (steps 3-5) or (x, y, w, h, d, t, u, v) (steps 6-8;
        step 8 applies it inside the next update, after copy())."""
        if len(rest) == 2:
            t, (u, v) = 0.0, rest
        elif len(rest) == 3:
            t, u, v = rest
        else:
            raise TypeError("addInflow(x, y, w, h, d, [t,] u, v)")
        self._check(self._L.ifl_add_inflow(self._h, x, y, w, h, d, t, u, v), "addInflow")

    def update(self, timestep: float):
        self._sync_bodies()
        self._check(self._L.ifl_update(self._h, timestep), "update")

    def ambientT(self) -> float:
        return float(self._L.ifl_ambient_t(self._h))

    # -- additions: readback, phases, statistics
    def run_phase(self, phase: int, timestep: float):
        self._sync_bodies()
        self._check(self._L.ifl_run_phase(self._h, phase, timestep), "run_phase")

    def shape(self, field: int):
        w, h = C.c_int(), C.c_int()
        self._check(self._L.ifl_field_shape(self._h, field, C.byref(w), C.byref(h)), "field_shape")
        return h.value, w.value

    def read_field(self, field, dtype=np.float64, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Copy a field to the host (into `out` when given, e.g. a pinned buffer)."""
        fid = _NAMED[field] if isinstance(field, str) else int(field)
        h, w = self.shape(fid)
        if out is not None:
            if out.shape != (h, w) or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous array of the field's shape")
            arr, dtype = out, out.dtype
        else:
            arr = np.empty((h, w), dtype=dtype)
        code = {np.dtype(np.float64): DT_F64, np.dtype(np.float32): DT_F32, np.dtype(np.uint8): DT_U8}[
            np.dtype(dtype)]
        self._check(self._L.ifl_read_field(self._h, fid, arr.ctypes.data, arr.nbytes, code), "read_field")
        return arr

    def write_field(self, field, values: np.ndarray):
        fid = _NAMED[field] if isinstance(field, str) else int(field)
        h, w = self.shape(fid)
        arr = np.ascontiguousarray(values)
        if arr.shape != (h, w):
            raise ValueError(f"field {fid}: expected shape {(h, w)}, got {arr.shape}")
        code = {np.dtype(np.float64): DT_F64, np.dtype(np.float32): DT_F32, np.dtype(np.uint8): DT_U8}[
            arr.dtype]
        self._check(self._L.ifl_write_field(self._h, fid, arr.ctypes.data, arr.nbytes, code), "write_field")

    def to_image(self, heat: bool = False) -> np.ndarray:
        """FluidSolver::toImage as an (h, w', 4) uint8 array (w' = 2w with heat in steps 6-8)."""
        wide = 2 if (heat and self.variant >= HEAT) else 1
        out = np.empty((self.h, wide * self.w, 4), dtype=np.uint8)
        self._check(self._L.ifl_render(self._h, 1 if heat else 0, out.ctypes.data, out.nbytes, 0), "to_image")
        return out

    def render_device(self, heat: bool, dev_ptr: int, nbytes: int):
        """toImage into device memory (asynchronous on the solver's stream)."""
        self._check(self._L.ifl_render(self._h, 1 if heat else 0, dev_ptr, nbytes, 1), "render_device")

    def flip(self, quantity: int):
        self._check(self._L.ifl_flip(self._h, quantity), "flip")

    # ---- step 8 (FLIP) particles
    def flip_init(self):
        """Place the initial particles now (the first update does it otherwise)."""
        self._sync_bodies()
        self._check(self._L.ifl_flip_init(self._h), "flip_init")

    def particle_count(self) -> int:
        n = C.c_int()
        self._check(self._L.ifl_particle_count(self._h, C.byref(n)), "particle_count")
        return n.value

    def particles(self, which: int) -> np.ndarray:
        """One particle array (P_X, P_Y, P_D, P_T, P_U, P_V) of the live particles."""
        cap = self.w * self.h * 12
        out = np.empty(cap, dtype=np.float64)
        n = C.c_int()
        self._check(self._L.ifl_read_particles(self._h, which, out.ctypes.data, cap, C.byref(n)), "particles")
        return out[:n.value].copy()

    def set_particles(self, arrays):
        """Replace the particle state: arrays = (x, y, d, t, u, v) of equal length."""
        n = len(arrays[0])
        for k, a in enumerate(arrays):
            a = np.ascontiguousarray(a, dtype=np.float64)
            if len(a) != n:
                raise ValueError("particle arrays differ in length")
            self._check(self._L.ifl_write_particles(self._h, k, a.ctypes.data, n), "set_particles")
        self._check(self._L.ifl_set_particle_count(self._h, n), "set_particles")

    @property
    def rng_state(self) -> int:
        v = C.c_uint32()
        self._check(self._L.ifl_get_rng_state(self._h, C.byref(v)), "rng_state")
        return int(v.value)

    @rng_state.setter
    def rng_state(self, value: int):
        self._check(self._L.ifl_set_rng_state(self._h, int(value) & 0xFFFFFFFF), "rng_state")

    def set_pinned_iterations(self, pressure: int, heat: int = -1):
        """-1: stop on the residual test; k >= 0: run exactly k PCG iterations."""
        self._check(self._L.ifl_set_pinned_iterations(self._h, pressure, heat), "pinned")

    def set_wait_limit(self, polls: int):
        """Polls of one device-side wait before the solve reports IFL_ERR_TIMEOUT (0: about a second)."""
        self._check(self._L.ifl_set_wait_limit(self._h, int(polls)), "wait_limit")

    def stats(self):
        st = StepStats()
        self._check(self._L.ifl_get_stats(self._h, C.byref(st)), "stats")
        return ((st.pressure.iterations, st.pressure.status, st.pressure.max_error),
                (st.heat.iterations, st.heat.status, st.heat.max_error), st.device_flags)

    def set_timing(self, on: bool = True):
        self._check(self._L.ifl_set_timing(self._h, 1 if on else 0), "set_timing")

    def timing(self):
        """Device ms and launches per kernel group since the last call, and PCG iterations."""
        t = Timing()
        self._check(self._L.ifl_get_timing(self._h, C.byref(t)), "get_timing")
        return ({n: t.ms[k] for k, n in enumerate(K_NAMES)},
                {n: int(t.launches[k]) for k, n in enumerate(K_NAMES)}, int(t.pcg_iterations))

    def synchronize(self):
        self._check(self._L.ifl_synchronize(self._h), "synchronize")

    @property
    def stream(self) -> int:
        return self._L.ifl_stream(self._h) or 0

    def launch_count(self) -> int:
        """Kernel launches this solver has issued since it was created."""
        return int(self._L.ifl_launch_count(self._h))


def plan_teams(grid: int, strips_per_block: int, strips, work):
    """ifl_batch_plan_teams: (blocks used, teams per class c = teams of 2**c blocks)."""
    L = load_library()
    n = len(strips)
    s_ = (C.c_int * n)(*[int(v) for v in strips])
    w_ = (C.c_double * n)(*[float(v) for v in work])
    t_ = (C.c_int * 8)()
    rc = L.ifl_batch_plan_teams(int(grid), int(strips_per_block), n, s_, w_, t_)
    if rc < 0:
        raise IflError(rc, "ifl_batch_plan_teams failed")
    return rc, list(t_)


class Batch:
    """Many FluidSolver handles advanced together (ifl_batch_*).

    ``Batch(solvers)`` groups handles of one variant, precision and device;
    ``set_inflows(i, [(x, y, w, h, d, u, v), ...])`` gives member i the
    rectangles it receives before every step (addInflow arguments, with t
    inserted for steps 6-7); ``update(dt)`` advances every member by one
    update() and returns when the step is complete.  Members keep their own
    bodies (moved with SolidBody.update between steps as usual) and stay
    ordinary handles between steps.
    """

    def __init__(self, solvers: Sequence[FluidSolver], threads: int = 0, strips_per_block: int = 0,
                 stages: int = 0, use_graph: bool = True, tune_iterations: int = 8, max_team_blocks: int = 0,
                 tiles=None):
        self._L = load_library()
        self.solvers = list(solvers)
        o = BatchOptions()
        self._L.ifl_batch_default_options(C.byref(o))
        o.threads, o.strips_per_block, o.stages = int(threads), int(strips_per_block), int(stages)
        o.use_graph = 1 if use_graph else 0
        o.tune_iterations = int(tune_iterations)
        o.max_team_blocks = int(max_team_blocks)
        # tiles: None = tune at the first update; "default" = 32 x 8; or a
        # {phase name: (threads, rows)} dict (phases not named: 32 x 8)
        if tiles is None:
            o.tile_tune = 1
        elif tiles == "default":
            o.tile_tune = 0
        else:
            o.tile_tune = 2
            for k, name in enumerate(TILE_PHASES):
                o.tile_w[k], o.tile_h[k] = tiles.get(name, (32, 8))
        arr = (C.c_void_p * len(self.solvers))(*[s._h for s in self.solvers])
        h_ = C.c_void_p()
        rc = self._L.ifl_batch_create(arr, len(self.solvers), C.byref(o), C.byref(h_))
        if rc != OK:
            msg = self._L.ifl_batch_last_error(None)
            raise IflError(rc, f"ifl_batch_create failed: {msg.decode() if msg else ''}")
        self._h = h_

    def close(self):
        if getattr(self, "_h", None):
            self._L.ifl_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != OK:
            msg = self._L.ifl_batch_last_error(self._h)
            raise IflError(rc, f"{what}: {msg.decode() if msg else ''}")

    def set_inflows(self, member: int, rects):
        rs = list(rects)
        arr = (Inflow * max(1, len(rs)))()
        for k, r in enumerate(rs):
            if len(r) == 7:
                x, y, w, h, d, u, v = r
                t = 0.0
            else:
                x, y, w, h, d, t, u, v = r
            arr[k] = Inflow(x, y, w, h, d, t, u, v)
        self._check(self._L.ifl_batch_set_inflows(self._h, int(member), arr, len(rs)), "set_inflows")

    def update(self, timestep: float):
        for s in self.solvers:
            s._sync_bodies()
        self._check(self._L.ifl_batch_update(self._h, float(timestep)), "batch update")

    def stats(self):
        n = len(self.solvers)
        arr = (StepStats * n)()
        self._check(self._L.ifl_batch_get_stats(self._h, arr, n), "batch stats")
        return [((a.pressure.iterations, a.pressure.status, a.pressure.max_error),
                 (a.heat.iterations, a.heat.status, a.heat.max_error), a.device_flags) for a in arr]

    def info(self) -> dict:
        o = BatchInfo()
        self._check(self._L.ifl_batch_get_info(self._h, C.byref(o)), "batch info")
        return {"members": o.members, "threads": o.threads, "strips_per_block": o.strips_per_block,
                "stages": o.stages, "grid": o.grid, "graph": bool(o.graph),
                "candidate_ms": [o.candidate_ms[k] for k in range(min(o.candidates, 8))],
                "last_step_ms": o.last_step_ms, "last_pcg_ms": o.last_pcg_ms,
                "launches": int(o.launches), "steps": int(o.steps),
                "h2d_bytes_last_step": int(o.h2d_bytes_last_step),
                "d2h_bytes_last_step": int(o.d2h_bytes_last_step),
                "tiles": {name: (o.tile_w[k], o.tile_h[k]) for k, name in enumerate(TILE_PHASES)},
                "tile_ms": {name: o.tile_ms[k] for k, name in enumerate(TILE_PHASES[:5]) if o.tile_ms[k] > 0}}

    @property
    def stream(self) -> int:
        return self._L.ifl_batch_stream(self._h) or 0


def device_bytes(variant: int, w: int, h: int, precision: int = FP64) -> int:
    """Device bytes a FluidSolver of this variant, size and precision allocates."""
    L = load_library()
    p = Params()
    L.ifl_default_params(C.byref(p), variant, int(w), int(h))
    p.precision = precision
    n = int(L.ifl_device_bytes(C.byref(p)))
    if n < 0:
        raise IflError(n, "ifl_device_bytes failed")
    return n


class Server:
    """Continuous-batching request loop (ifl_server_*).

    ``submit(w, h, steps, bodies=(), inflows=(), arrival=None)`` queues a
    scene; ``step()`` admits what fits and advances every admitted request by
    one update(); ``completions()`` lists requests finished since the last
    call; ``read_field(id, name)`` reads a finished request's field and
    ``release(id)`` frees its device state.
    """

    def __init__(self, variant: int = SOLID, precision: int = FP32, device: int = 0, dt: float = 0.0025,
                 hbm_budget_bytes: int = 0, max_active: int = 1024, dry_run: bool = False, threads: int = 0,
                 strips_per_block: int = 0, stages: int = 0, use_graph: bool = True):
        self._L = load_library()
        p = ServerParams()
        self._L.ifl_server_default_params(C.byref(p), variant, precision)
        p.device, p.dt, p.hbm_budget_bytes, p.max_active = int(device), float(dt), int(hbm_budget_bytes), int(max_active)
        p.dry_run = 1 if dry_run else 0
        p.batch.threads, p.batch.strips_per_block, p.batch.stages = int(threads), int(strips_per_block), int(stages)
        p.batch.use_graph = 1 if use_graph else 0
        h_ = C.c_void_p()
        rc = self._L.ifl_server_create(C.byref(p), C.byref(h_))
        if rc != OK:
            raise IflError(rc, "ifl_server_create failed")
        self._h = h_
        self.variant, self.precision = variant, precision

    def close(self):
        if getattr(self, "_h", None):
            self._L.ifl_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != OK:
            msg = self._L.ifl_server_last_error(self._h)
            raise IflError(rc, f"{what}: {msg.decode() if msg else ''}")

    def now(self) -> float:
        return float(self._L.ifl_server_now(self._h))

    def submit(self, w: int, h: int, steps: int, bodies=(), inflows=(), arrival=None) -> int:
        bl = [_body_tuple(b) for b in bodies]
        barr = (_CBody * max(1, len(bl)))()
        for k, b in enumerate(bl):
            barr[k].type = int(b[0])
            (barr[k].pos_x, barr[k].pos_y, barr[k].scale_x, barr[k].scale_y, barr[k].theta, barr[k].vel_x,
             barr[k].vel_y, barr[k].vel_theta) = [float(x) for x in b[1:9]]
        il = list(inflows)
        iarr = (Inflow * max(1, len(il)))()
        for k, r in enumerate(il):
            if len(r) == 7:
                x, y, ww, hh, dd, u, v = r
                t = 0.0
            else:
                x, y, ww, hh, dd, t, u, v = r
            iarr[k] = Inflow(x, y, ww, hh, dd, t, u, v)
        r = Request(int(w), int(h), int(steps), len(bl), len(il), 0, C.cast(barr, C.c_void_p),
                    C.cast(iarr, C.c_void_p), float(self.now() if arrival is None else arrival))
        rid = C.c_int64(0)
        self._check(self._L.ifl_server_submit(self._h, C.byref(r), C.byref(rid)), "submit")
        return int(rid.value)

    def step(self):
        a, q = C.c_int(0), C.c_int(0)
        self._check(self._L.ifl_server_step(self._h, C.byref(a), C.byref(q)), "step")
        return a.value, q.value

    def completions(self):
        out = []
        buf = (Completion * 256)()
        while True:
            n = C.c_int(0)
            self._check(self._L.ifl_server_completions(self._h, buf, 256, C.byref(n)), "completions")
            out += [{"id": c.id, "w": c.w, "h": c.h, "steps": c.steps, "arrival": c.arrival,
                     "admitted": c.admitted, "finished": c.finished, "device_bytes": c.device_bytes}
                    for c in buf[:n.value]]
            if n.value < 256:
                return out

    def read_field(self, rid: int, field, dtype=np.float64) -> np.ndarray:
        """Copy a field of an admitted or finished request to the host."""
        f = _NAMED[field] if isinstance(field, str) else int(field)
        w, h = C.c_int(), C.c_int()
        self._check(self._L.ifl_server_field_shape(self._h, rid, f, C.byref(w), C.byref(h)), "field_shape")
        out = np.empty((h.value, w.value), dtype=dtype)
        code = {np.dtype(np.float64): DT_F64, np.dtype(np.float32): DT_F32, np.dtype(np.uint8): DT_U8}[np.dtype(dtype)]
        self._check(self._L.ifl_server_read_field(self._h, rid, f, out.ctypes.data, out.nbytes, code), "read_field")
        return out

    def stats(self, rid: int):
        st = StepStats()
        self._check(self._L.ifl_server_request_stats(self._h, rid, C.byref(st)), "stats")
        return ((st.pressure.iterations, st.pressure.status, st.pressure.max_error),
                (st.heat.iterations, st.heat.status, st.heat.max_error), st.device_flags)

    def release(self, rid: int):
        self._check(self._L.ifl_server_release(self._h, rid), "release")

    def info(self) -> dict:
        o = ServerInfo()
        self._check(self._L.ifl_server_get_info(self._h, C.byref(o)), "info")
        return {k: getattr(o, k) for k, _ in ServerInfo._fields_ if k != "pad_"}


def write_png(path: str, rgba: np.ndarray):
    """Write an (h, w, 4) uint8 RGBA image as a PNG file (8-bit RGBA, no filtering),
    rows in array order as lodepng_encode32_file writes the reference's frames."""
    import struct
    import zlib
    img = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w, _ = img.shape
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(kind: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))
