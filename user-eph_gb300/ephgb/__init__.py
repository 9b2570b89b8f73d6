"""Python side of the GB300 fix-eph path: ctypes bindings of libephgb.so (the
C ABI in include/eph_gb.h) and `FixEPH`, a mirror of the LAMMPS fix `eph`
interface (fix_eph.h:62-83) built from the same fix words.

The library is the only compute path: importing works without a GPU (the
host-side beta/grid helpers run on the CPU), but every hook raises if the
CUDA library cannot be loaded or the device call fails.  There is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import workloads  # noqa: F401

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(ROOT, "libephgb.so")

EPH_OK = 0
STATUS = {0: "EPH_OK", 1: "EPH_ERR_ARG", 2: "EPH_ERR_FILE", 3: "EPH_ERR_UNSUPPORTED_MODEL", 4: "EPH_ERR_CAPACITY",
          5: "EPH_ERR_TIMEOUT", 6: "EPH_ERR_CUDA", 7: "EPH_ERR_STATE", 8: "EPH_ERR_RANGE"}
MODE_EXACT, MODE_FAST = 0, 1
PAIRS_FP64, PAIRS_DF64 = 0, 1
HOST, DEVICE, HOST_ASYNC = 0, 1, 2
XI_DEVICE_RNG, XI_GIVEN = 0, 1
FIELDS = {"x": (0, 3), "v": (1, 3), "f": (2, 3), "xi": (3, 3), "f_eph": (4, 3), "f_rng": (5, 3), "rho": (6, 1),
          "w": (7, 3), "array": (8, 8), "T": (9, None), "f_ext": (10, 3)}
SPLINES = {"rho_r": 0, "rho_r_sq": 1, "beta": 2, "alpha": 3}
COUNTERS = {"rho_cutoff": 0, "T_clamp": 1, "build": 2, "wrap": 3}
PHASES = ("integrate", "bin", "density", "friction_w", "forces", "deposit", "fdm", "pair")


class EphError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class eph_md(C.Structure):
    _fields_ = [("ntypes", C.c_int), ("mass", C.POINTER(C.c_double)), ("boxlo", C.c_double * 3),
                ("boxhi", C.c_double * 3), ("dt", C.c_double), ("boltz", C.c_double), ("ftm2v", C.c_double),
                ("skin", C.c_double), ("groupbit", C.c_int), ("device", C.c_int), ("mode", C.c_int)]


_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# name -> (restype, argtypes); mirrors include/eph_gb.h
SIGNATURES = {
    "eph_create": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), C.POINTER(eph_md), C.POINTER(C.c_void_p)]),
    "eph_destroy": (None, [C.c_void_p]),
    "eph_last_error": (C.c_char_p, [C.c_void_p]),
    "eph_status_string": (C.c_char_p, [C.c_int]),
    "eph_set_atoms": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _ip, _ip]),
    "eph_put": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "eph_get": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "eph_initial_integrate": (C.c_int, [C.c_void_p]),
    "eph_post_force": (C.c_int, [C.c_void_p, C.c_int]),
    "eph_final_integrate": (C.c_int, [C.c_void_p]),
    "eph_end_of_step": (C.c_int, [C.c_void_p]),
    "eph_step": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "eph_compute_vector": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "eph_reset_dt": (C.c_int, [C.c_void_p, C.c_double]),
    "eph_save_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "eph_save_temperature": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "eph_post_run": (C.c_int, [C.c_void_p]),
    "eph_set_timestep": (C.c_int, [C.c_void_p, C.c_long]),
    "eph_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "eph_synchronize": (C.c_int, [C.c_void_p]),
    "eph_get_counter": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_long)]),
    "eph_set_capacity": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "eph_set_graph": (C.c_int, [C.c_void_p, C.c_int]),
    "eph_set_pair_eam": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_char_p)]),
    "eph_pair_energy": (C.c_int, [C.c_void_p, _dp]),
    "eph_set_threads_per_atom": (C.c_int, [C.c_void_p, C.c_int]),
    "eph_set_pair_arithmetic": (C.c_int, [C.c_void_p, C.c_int]),
    "eph_get_threads_per_atom": (C.c_int, [C.c_void_p, _ip]),
    "eph_set_list_skin": (C.c_int, [C.c_void_p, C.c_double]),
    "eph_get_list_skin": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), _ip]),
    "eph_autotune": (C.c_int, [C.c_void_p, _ip]),
    "eph_initial_integrate_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "eph_post_force_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "eph_final_integrate_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "eph_pin": (C.c_int, [C.c_void_p, C.c_size_t]),
    "eph_unpin": (C.c_int, [C.c_void_p]),
    "eph_autotune_list_skin": (C.c_int, [C.c_void_p, _dp, C.c_int, C.c_int, _dp]),
    "eph_batch_create": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.POINTER(C.c_char_p)),
                                   C.POINTER(eph_md), C.POINTER(C.c_void_p)]),
    "eph_batch_destroy": (None, [C.c_void_p]),
    "eph_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "eph_batch_set_atoms": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _ip, _ip]),
    "eph_batch_step": (C.c_int, [C.c_void_p, C.c_int]),
    "eph_batch_synchronize": (C.c_int, [C.c_void_p]),
    "eph_batch_context": (C.c_void_p, [C.c_void_p, C.c_int]),
    "eph_batch_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_long)]),
    "eph_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "eph_phase_times": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_long)]),
    "eph_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_long)]),
    "eph_pair_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_long)]),
    "eph_fdm_solve_noalloc": (C.c_int, [C.c_long, C.c_long, C.c_long, _dp, _dp, C.c_double, C.c_long, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.POINTER(C.c_uint)]),
    "eph_beta_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "eph_beta_free": (None, [C.c_void_p]),
    "eph_beta_info": (C.c_int, [C.c_void_p, _ip, _dp, _dp]),
    "eph_beta_eval": (C.c_double, [C.c_void_p, C.c_int, C.c_int, C.c_double]),
    "eph_beta_table": (C.c_long, [C.c_void_p, C.c_int, C.c_int, _dp]),
    "eph_grid_create": (C.c_int, [C.c_long, C.c_long, C.c_long, _dp, _dp, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.POINTER(C.c_void_p)]),
    "eph_grid_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "eph_grid_free": (None, [C.c_void_p]),
    "eph_grid_ncells": (C.c_long, [C.c_void_p]),
    "eph_grid_substeps": (C.c_uint, [C.c_void_p, C.c_double, _dp]),
    "eph_grid_save_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "eph_grid_save_temperature": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "eph_beta_set_knots": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_long, _dp, C.c_long]),
    "eph_beta_knot_gradient": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]),
    "eph_set_beta_knots": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_long, _dp, C.c_long]),
    "eph_set_grid_constants": (C.c_int, [C.c_void_p, C.c_double, C.c_double]),
    "eph_adjoint_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "eph_adjoint_destroy": (None, [C.c_void_p]),
    "eph_adjoint_last_error": (C.c_char_p, [C.c_void_p]),
    "eph_adjoint_forward": (C.c_int, [C.c_void_p, C.c_long, _dp, _dp]),
    "eph_adjoint_backward": (C.c_int, [C.c_void_p, _dp, _dp]),
    "eph_adjoint_gradient": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_long]),
    "eph_adjoint_set_graph": (C.c_int, [C.c_void_p, C.c_int]),
    "eph_adjoint_batch_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "eph_adjoint_batch_destroy": (None, [C.c_void_p]),
    "eph_adjoint_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "eph_adjoint_batch_forward": (C.c_int, [C.c_void_p, C.c_long, _dp, _dp]),
    "eph_adjoint_batch_backward": (C.c_int, [C.c_void_p, _dp, _dp]),
    "eph_adjoint_batch_timing": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    "eph_adjoint_timing": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_long), C.POINTER(C.c_long)]),
}


def lib():
    """Load libephgb.so (raises if it was not built: no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run __graft_entry__.build() (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class BetaFile:
    """Host-side beta(rho) file and its splines (eph_beta.h:39-198)."""

    def __init__(self, path):
        L = lib()
        h = C.c_void_p()
        rc = L.eph_beta_load(path.encode(), C.byref(h))
        if rc:
            raise EphError(rc, f"cannot load {path}")
        self.h = h
        n = C.c_int()
        r = C.c_double()
        rho = C.c_double()
        L.eph_beta_info(h, C.byref(n), C.byref(r), C.byref(rho))
        self.n_elements, self.r_cutoff, self.rho_cutoff = n.value, r.value, rho.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().eph_beta_free(self.h)
            self.h = None

    def eval(self, which, elem, x):
        L = lib()
        w = SPLINES[which]
        return np.array([L.eph_beta_eval(self.h, w, elem, float(v)) for v in np.atleast_1d(x)])

    def table(self, which, elem):
        L = lib()
        w = SPLINES[which]
        n = L.eph_beta_table(self.h, w, elem, None)
        out = np.zeros((n, 4))
        L.eph_beta_table(self.h, w, elem, out.ctypes.data_as(_dp))
        return out

    def set_knots(self, elem, rho_knots, beta_knots):
        r = np.ascontiguousarray(rho_knots, dtype=np.float64)
        b = np.ascontiguousarray(beta_knots, dtype=np.float64)
        rc = lib().eph_beta_set_knots(self.h, elem, r.ctypes.data_as(_dp), r.size, b.ctypes.data_as(_dp), b.size)
        if rc:
            raise EphError(rc, "knot columns do not match the file")

    def knot_gradient(self, elem, g_rho_r_sq, g_alpha):
        """dL/d(rho(r) knots), dL/d(beta knots) from dL/d(coefficients) of the
        rho(r^2) and alpha tables (arrays of n x 4)."""
        gr = np.ascontiguousarray(g_rho_r_sq, dtype=np.float64)
        ga = np.ascontiguousarray(g_alpha, dtype=np.float64)
        out_r = np.zeros(gr.size // 4)
        out_b = np.zeros(ga.size // 4)
        rc = lib().eph_beta_knot_gradient(self.h, elem, gr.ctypes.data_as(_dp), ga.ctypes.data_as(_dp),
                                          out_r.ctypes.data_as(_dp), out_b.ctypes.data_as(_dp))
        if rc:
            raise EphError(rc, "knot_gradient")
        return out_r, out_b


class Grid:
    """Host-side electronic grid: uniform or read from a grid file."""

    def __init__(self, path=None, n=None, lo=None, hi=None, T_e=300.0, C_e=3.5e-6, rho_e=1.0, kappa_e=0.1):
        L = lib()
        h = C.c_void_p()
        if path is not None:
            rc = L.eph_grid_load(path.encode(), C.byref(h))
        else:
            lo = np.ascontiguousarray(lo, dtype=np.float64)
            hi = np.ascontiguousarray(hi, dtype=np.float64)
            rc = L.eph_grid_create(n[0], n[1], n[2], lo.ctypes.data_as(_dp), hi.ctypes.data_as(_dp), T_e, C_e,
                                   rho_e, kappa_e, C.byref(h))
        if rc:
            raise EphError(rc, "cannot build grid")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().eph_grid_free(self.h)
            self.h = None

    @property
    def ncells(self):
        return lib().eph_grid_ncells(self.h)

    def substeps(self, dt):
        idt = C.c_double()
        n = lib().eph_grid_substeps(self.h, dt, C.byref(idt))
        return n, idt.value

    def save_state(self, path):
        rc = lib().eph_grid_save_state(self.h, path.encode())
        if rc:
            raise EphError(rc, path)

    def save_temperature(self, path, n):
        rc = lib().eph_grid_save_temperature(self.h, path.encode(), n)
        if rc:
            raise EphError(rc, path)


class FixEPH:
    """The fix `eph` on one GPU, built from the fix command's words.

    Mirrors FixEPH (fix_eph.h:62-83): initial_integrate, post_force,
    final_integrate, end_of_step, compute_vector, reset_dt, post_run, the
    per-atom array (`array_atom`), plus `step(n)` which runs n engine steps
    device-resident."""

    def __init__(self, words, atoms=None, dt=0.001, mass=None, boxlo=None, boxhi=None, skin=1.0,
                 boltz=workloads.BOLTZ, ftm2v=workloads.FTM2V, groupbit=1, device=0, mode=MODE_FAST, eam=None):
        L = lib()
        self.L = L
        if atoms is not None:
            mass = atoms.mass if mass is None else mass
            boxlo = atoms.boxlo if boxlo is None else boxlo
            boxhi = atoms.boxhi if boxhi is None else boxhi
        self._mass = np.ascontiguousarray(mass, dtype=np.float64)
        md = eph_md()
        md.ntypes = len(self._mass) - 1
        md.mass = self._mass.ctypes.data_as(_dp)
        for k in range(3):
            md.boxlo[k] = float(boxlo[k])
            md.boxhi[k] = float(boxhi[k])
        md.dt, md.boltz, md.ftm2v, md.skin = dt, boltz, ftm2v, skin
        md.groupbit, md.device, md.mode = groupbit, device, mode
        self.words = [str(w) for w in words]
        self._argv = (C.c_char_p * len(words))(*[w.encode() for w in words])
        h = C.c_void_p()
        rc = L.eph_create(len(words), self._argv, C.byref(md), C.byref(h))
        self.h = h
        self._check(rc)
        self.n = 0
        self.ncells = grid_cells(words)
        if eam is not None:  # (setfl path, [element per type])
            self.set_pair_eam(*eam)
        if atoms is not None:
            self.set_atoms(atoms.x, atoms.v, atoms.type, atoms.mask)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.eph_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc != EPH_OK:
            msg = self.L.eph_last_error(self.h).decode() if getattr(self, "h", None) else ""
            raise EphError(rc, msg)

    def set_atoms(self, x, v, type_, mask=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        t = np.ascontiguousarray(type_, dtype=np.int32)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        self._check(self.L.eph_set_atoms(self.h, x.shape[0], x.ctypes.data_as(_dp), v.ctypes.data_as(_dp),
                                         t.ctypes.data_as(_ip), None if m is None else m.ctypes.data_as(_ip)))
        self.n = x.shape[0]

    # ---- data movement
    def put(self, field, arr, asynchronous=False):
        """asynchronous: the copy is queued; `arr` (a contiguous float64
        array, ideally pinned) must stay unchanged until the next
        synchronising call"""
        fid, _ = FIELDS[field]
        if hasattr(arr, "data_ptr"):  # torch tensor on the device
            self._check(self.L.eph_put(self.h, fid, C.c_void_p(arr.data_ptr()), DEVICE))
            return
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if asynchronous and a is not arr:
            raise ValueError("an asynchronous put needs a contiguous float64 array")
        self._check(self.L.eph_put(self.h, fid, _ptr(a), HOST_ASYNC if asynchronous else HOST))

    def get_async(self, field, out):
        """queue a copy into `out` (contiguous float64, ideally pinned); it
        is complete after the next synchronising call"""
        fid, _ = FIELDS[field]
        self._check(self.L.eph_get(self.h, fid, _ptr(out), HOST_ASYNC))
        return out

    def get(self, field, out=None):
        fid, k = FIELDS[field]
        if out is not None and hasattr(out, "data_ptr"):
            self._check(self.L.eph_get(self.h, fid, C.c_void_p(out.data_ptr()), DEVICE))
            return out
        if field == "T":
            shape = (self.ncells,)
        else:
            shape = (self.n, k) if k > 1 else (self.n,)
        a = np.zeros(shape) if out is None else out
        self._check(self.L.eph_get(self.h, fid, _ptr(a), HOST))
        return a

    # ---- hooks
    def initial_integrate(self):
        self._check(self.L.eph_initial_integrate(self.h))

    def post_force(self, xi=None):
        if xi is not None:
            self.put("xi", xi)
            self._check(self.L.eph_post_force(self.h, XI_GIVEN))
        else:
            self._check(self.L.eph_post_force(self.h, XI_DEVICE_RNG))

    def final_integrate(self):
        self._check(self.L.eph_final_integrate(self.h))

    def end_of_step(self):
        self._check(self.L.eph_end_of_step(self.h))

    # the hooks with the engine's host arrays (contiguous float64 n x 3,
    # ideally pinned), in place; equal to put / hook / get with overlapped
    # copies
    def _rows(self, a, k=3):
        if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous
                and a.shape == (self.n, k)):
            raise ValueError(f"expected a C-contiguous float64 array of shape ({self.n}, {k})")
        return _ptr(a)

    def initial_integrate_host(self, x, v):
        self._check(self.L.eph_initial_integrate_host(self.h, self._rows(x), self._rows(v)))

    def post_force_host(self, x, f, array=None, xi=None, f_in=None):
        """x: positions to upload (None: the device's), f: the engine's force
        in (or f_in when given), the total out; array (n x 8): the per-atom
        array, written by the time end_of_step returns"""
        if xi is not None:
            self.put("xi", xi)
        fi = self._rows(f if f_in is None else f_in)
        self._check(self.L.eph_post_force_host(self.h, None if x is None else self._rows(x), fi, self._rows(f),
                                               None if array is None else self._rows(array, 8),
                                               XI_GIVEN if xi is not None else XI_DEVICE_RNG))

    def final_integrate_host(self, f, v):
        self._check(self.L.eph_final_integrate_host(self.h, self._rows(f), self._rows(v)))

    def step(self, nsteps=1, xi=None):
        """nsteps engine steps; xi (n x 3) feeds the deviates of a single step."""
        if xi is not None:
            self.put("xi", xi)
            self._check(self.L.eph_step(self.h, nsteps, XI_GIVEN))
        else:
            self._check(self.L.eph_step(self.h, nsteps, XI_DEVICE_RNG))

    def compute_vector(self, i):
        out = C.c_double()
        self._check(self.L.eph_compute_vector(self.h, i, C.byref(out)))
        return out.value

    @property
    def array_atom(self):
        return self.get("array")

    def reset_dt(self, dt):
        self._check(self.L.eph_reset_dt(self.h, dt))

    def save_state(self, path):
        self._check(self.L.eph_save_state(self.h, path.encode()))

    def save_temperature(self, path, n):
        self._check(self.L.eph_save_temperature(self.h, path.encode(), n))

    def post_run(self):
        self._check(self.L.eph_post_run(self.h))

    def synchronize(self):
        self._check(self.L.eph_synchronize(self.h))

    def counter(self, name):
        out = C.c_long()
        self._check(self.L.eph_get_counter(self.h, COUNTERS[name], C.byref(out)))
        return out.value

    def set_capacity(self, bins=0, pairs=0):
        self._check(self.L.eph_set_capacity(self.h, bins, pairs))

    def set_profiling(self, on=True):
        self._check(self.L.eph_set_profiling(self.h, 1 if on else 0))

    def phase_times(self):
        ms = np.zeros(len(PHASES))
        n = (C.c_long * len(PHASES))()
        self._check(self.L.eph_phase_times(self.h, ms.ctypes.data_as(_dp), n))
        return {p: (ms[k], n[k]) for k, p in enumerate(PHASES)}

    def launch_count(self):
        out = C.c_long()
        self._check(self.L.eph_launch_count(self.h, C.byref(out)))
        return out.value

    def pair_count(self):
        out = C.c_long()
        self._check(self.L.eph_pair_count(self.h, C.byref(out)))
        return out.value

    def set_stream(self, stream_ptr):
        self._check(self.L.eph_set_stream(self.h, C.c_void_p(stream_ptr)))

    def set_graph(self, on=True):
        self._check(self.L.eph_set_graph(self.h, 1 if on else 0))

    def set_pair_eam(self, path, elements):
        """eam/alloy pair force for eph_step (call before set_atoms)"""
        arr = (C.c_char_p * len(elements))(*[e.encode() for e in elements])
        self._check(self.L.eph_set_pair_eam(self.h, path.encode(), len(elements), arr))

    def pair_energy(self):
        out = C.c_double()
        self._check(self.L.eph_pair_energy(self.h, C.byref(out)))
        return out.value

    def set_threads_per_atom(self, tpa):
        self._check(self.L.eph_set_threads_per_atom(self.h, int(tpa)))

    def set_pair_arithmetic(self, which):
        """PAIRS_DF64 (default) or PAIRS_FP64: the FAST one-lane pair sweeps'
        per-pair arithmetic (eph_set_pair_arithmetic)."""
        self._check(self.L.eph_set_pair_arithmetic(self.h, int(which)))

    def threads_per_atom(self):
        out = C.c_int()
        self._check(self.L.eph_get_threads_per_atom(self.h, C.byref(out)))
        return out.value

    def set_list_skin(self, skin):
        """Skin of the kept candidate lists (0 searches the bins every step)."""
        self._check(self.L.eph_set_list_skin(self.h, float(skin)))

    def list_skin(self):
        """(skin, whether the context keeps candidate lists)"""
        s, a = C.c_double(), C.c_int()
        self._check(self.L.eph_get_list_skin(self.h, C.byref(s), C.byref(a)))
        return s.value, bool(a.value)

    def autotune(self):
        out = C.c_int()
        self._check(self.L.eph_autotune(self.h, C.byref(out)))
        return out.value

    def autotune_list_skin(self, skins=(0.0, 0.2, 0.3, 0.5, 0.8), steps=20):
        """eph_autotune_list_skin: time `steps` steps from the current state
        with each skin (each window starting with a list build), restore the
        state and keep the fastest skin; returns it"""
        sk = np.ascontiguousarray(skins, dtype=np.float64)
        out = C.c_double()
        self._check(self.L.eph_autotune_list_skin(self.h, sk.ctypes.data_as(_dp), sk.size, int(steps),
                                                   C.byref(out)))
        return out.value

    def set_beta_knots(self, elem, rho_knots, beta_knots):
        r = np.ascontiguousarray(rho_knots, dtype=np.float64)
        b = np.ascontiguousarray(beta_knots, dtype=np.float64)
        self._check(lib().eph_set_beta_knots(self.h, elem, r.ctypes.data_as(_dp), r.size, b.ctypes.data_as(_dp),
                                             b.size))

    def set_grid_constants(self, C_e, kappa_e):
        self._check(lib().eph_set_grid_constants(self.h, float(C_e), float(kappa_e)))

    def set_timestep(self, n):
        self._check(self.L.eph_set_timestep(self.h, n))


class _View(FixEPH):
    """A replica's context owned by a Batch (not destroyed on its own)."""

    def __init__(self, L, h, words, n):
        self.L, self.h, self.n = L, h, n
        self.ncells = grid_cells(words)

    def __del__(self):
        pass


class Batch:
    """Batched replicas: independent fix instances stepped together, one
    CUDA-graph launch per step (eph_batch_* in include/eph_gb.h)."""

    def __init__(self, replicas, dt=0.001, skin=1.0, boltz=workloads.BOLTZ, ftm2v=workloads.FTM2V, device=0,
                 mode=MODE_FAST):
        """replicas: list of (words, atoms)."""
        L = lib()
        self.L = L
        R = len(replicas)
        self._keep = []
        mds = (eph_md * R)()
        argvs = (C.POINTER(C.c_char_p) * R)()
        nargs = (C.c_int * R)()
        for r, (words, atoms) in enumerate(replicas):
            mass = np.ascontiguousarray(atoms.mass, dtype=np.float64)
            argv = (C.c_char_p * len(words))(*[w.encode() for w in words])
            self._keep += [mass, argv]
            md = mds[r]
            md.ntypes = len(mass) - 1
            md.mass = mass.ctypes.data_as(_dp)
            for k in range(3):
                md.boxlo[k] = float(atoms.boxlo[k])
                md.boxhi[k] = float(atoms.boxhi[k])
            md.dt, md.boltz, md.ftm2v, md.skin = dt, boltz, ftm2v, skin
            md.groupbit, md.device, md.mode = 1, device, mode
            argvs[r] = C.cast(argv, C.POINTER(C.c_char_p))
            nargs[r] = len(words)
        h = C.c_void_p()
        rc = L.eph_batch_create(R, nargs, argvs, mds, C.byref(h))
        self.h = h
        if rc:
            msg = L.eph_batch_last_error(h).decode() if h else ""
            raise EphError(rc, msg)
        self.replicas = []
        for r, (words, atoms) in enumerate(replicas):
            x = np.ascontiguousarray(atoms.x, dtype=np.float64)
            v = np.ascontiguousarray(atoms.v, dtype=np.float64)
            t = np.ascontiguousarray(atoms.type, dtype=np.int32)
            m = np.ascontiguousarray(atoms.mask, dtype=np.int32)
            rc = L.eph_batch_set_atoms(h, r, atoms.n, x.ctypes.data_as(_dp), v.ctypes.data_as(_dp),
                                       t.ctypes.data_as(_ip), m.ctypes.data_as(_ip))
            if rc:
                raise EphError(rc, L.eph_batch_last_error(h).decode())
            self.replicas.append(_View(L, L.eph_batch_context(h, r), words, atoms.n))

    def __del__(self):
        if getattr(self, "h", None):
            self.replicas = []
            self.L.eph_batch_destroy(self.h)
            self.h = None

    def step(self, nsteps=1):
        rc = self.L.eph_batch_step(self.h, nsteps)
        if rc:
            raise EphError(rc, self.L.eph_batch_last_error(self.h).decode())

    def synchronize(self):
        rc = self.L.eph_batch_synchronize(self.h)
        if rc:
            raise EphError(rc, self.L.eph_batch_last_error(self.h).decode())

    def launches_per_step(self):
        out = C.c_long()
        self.L.eph_batch_launch_count(self.h, C.byref(out))
        return out.value


def grid_cells(words):
    """Number of grid cells a fix line defines (NX*NY*NZ for a NULL grid file,
    else read from the grid file)."""
    if words[13] == "NULL":
        return int(words[10]) * int(words[11]) * int(words[12])
    return Grid(path=words[13]).ncells
