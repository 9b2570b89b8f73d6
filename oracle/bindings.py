"""ctypes bindings of the CPU oracle (liboracle.so, the C restatement) and of
the reference fix compiled with the engine stand-in (_ref/libephref.so, only
where the reference tree was present at build time).  TEST INFRASTRUCTURE
ONLY."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libephref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _argv(words):
    arr = (C.c_char_p * len(words))(*[w.encode() for w in words])
    return arr


_orc = None


def oracle_lib():
    global _orc
    if _orc is None:
        lib = C.CDLL(ORACLE_SO)
        lib.orc_fix_create.restype = C.c_void_p
        lib.orc_fix_create.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_int, _dp, _dp, _dp, C.c_double,
                                       C.c_double, C.c_double, C.c_double, C.c_char_p, C.c_int]
        lib.orc_fix_free.argtypes = [C.c_void_p]
        lib.orc_fix_set_atoms.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _ip, _ip, C.c_int]
        lib.orc_fix_set_fext.argtypes = [C.c_void_p, _dp]
        lib.orc_fix_set_threads.argtypes = [C.c_void_p, C.c_int]
        lib.orc_fix_step.argtypes = [C.c_void_p, _dp]
        lib.orc_fix_get.argtypes = [C.c_void_p, C.c_char_p, _dp]
        lib.orc_fix_set.argtypes = [C.c_void_p, C.c_char_p, _dp]
        lib.orc_fix_nbuild.restype = C.c_long
        lib.orc_fix_nbuild.argtypes = [C.c_void_p]
        lib.orc_fix_neigh.argtypes = [C.c_void_p, _ip, _ip, C.c_int]
        lib.orc_fix_seconds.restype = C.c_double
        lib.orc_fix_seconds.argtypes = [C.c_void_p, C.c_int]
        lib.orc_fix_fdm.restype = C.c_void_p
        lib.orc_fix_fdm.argtypes = [C.c_void_p]
        lib.orc_fix_beta.restype = C.c_void_p
        lib.orc_fix_beta.argtypes = [C.c_void_p]
        lib.orc_beta_load.restype = C.c_void_p
        lib.orc_beta_load.argtypes = [C.c_char_p]
        lib.orc_beta_free.argtypes = [C.c_void_p]
        lib.orc_beta_eval.restype = C.c_double
        lib.orc_beta_eval.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
        lib.orc_beta_get_beta.restype = C.c_double
        lib.orc_beta_get_beta.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.orc_beta_get_alpha.restype = C.c_double
        lib.orc_beta_get_alpha.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.orc_beta_table.restype = C.c_long
        lib.orc_beta_table.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        lib.orc_beta_r_cutoff.restype = C.c_double
        lib.orc_beta_r_cutoff.argtypes = [C.c_void_p]
        lib.orc_beta_rho_cutoff.restype = C.c_double
        lib.orc_beta_rho_cutoff.argtypes = [C.c_void_p]
        lib.orc_fdm_create.restype = C.c_void_p
        lib.orc_fdm_create.argtypes = [C.c_long] * 3 + [C.c_double] * 10
        lib.orc_fdm_load.restype = C.c_void_p
        lib.orc_fdm_load.argtypes = [C.c_char_p]
        lib.orc_fdm_free.argtypes = [C.c_void_p]
        lib.orc_fdm_set_dt.argtypes = [C.c_void_p, C.c_double]
        lib.orc_fdm_insert_energy.argtypes = [C.c_void_p] + [C.c_double] * 4
        lib.orc_fdm_get_T.restype = C.c_double
        lib.orc_fdm_get_T.argtypes = [C.c_void_p] + [C.c_double] * 3
        lib.orc_fdm_get_T_total.restype = C.c_double
        lib.orc_fdm_get_T_total.argtypes = [C.c_void_p]
        lib.orc_fdm_get_index.restype = C.c_long
        lib.orc_fdm_get_index.argtypes = [C.c_void_p] + [C.c_double] * 3
        lib.orc_fdm_solve.restype = C.c_uint
        lib.orc_fdm_solve.argtypes = [C.c_void_p]
        lib.orc_fdm_save_state.argtypes = [C.c_void_p, C.c_char_p]
        lib.orc_fdm_save_temperature.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        lib.orc_fdm_ncells.restype = C.c_long
        lib.orc_fdm_ncells.argtypes = [C.c_void_p]
        lib.orc_fdm_get.argtypes = [C.c_void_p, C.c_int, _dp]
        lib.orc_fdm_set.argtypes = [C.c_void_p, C.c_int, _dp]
        lib.orc_ranmars_init_ijkl.argtypes = [C.c_void_p, C.c_int, C.c_int]
        lib.orc_ranmars_init.argtypes = [C.c_void_p, C.c_int]
        lib.orc_ranmars_uniform.restype = C.c_double
        lib.orc_ranmars_uniform.argtypes = [C.c_void_p]
        lib.orc_ranmars_gaussian.restype = C.c_double
        lib.orc_ranmars_gaussian.argtypes = [C.c_void_p]
        _orc = lib
    return _orc


class OracleFix:
    """The CPU restatement of the fix, driven like the engine drives it."""

    def __init__(self, words, atoms, dt, skin=1.0, boltz=8.617343e-5, ftm2v=1.0 / 1.0364269e-4, groupbit=1,
                 threads=1):
        lib = oracle_lib()
        self.lib = lib
        err = C.create_string_buffer(512)
        mass = np.ascontiguousarray(atoms.mass, dtype=np.float64)
        ntypes = len(mass) - 1
        self.h = lib.orc_fix_create(len(words), _argv(words), ntypes, _d(mass), _d(atoms.boxlo), _d(atoms.boxhi),
                                    dt, boltz, ftm2v, skin, err, 512)
        if not self.h:
            raise RuntimeError(err.value.decode())
        self.n = atoms.n
        lib.orc_fix_set_threads(self.h, threads)
        x = np.ascontiguousarray(atoms.x, dtype=np.float64)
        v = np.ascontiguousarray(atoms.v, dtype=np.float64)
        t = np.ascontiguousarray(atoms.type, dtype=np.int32)
        m = np.ascontiguousarray(atoms.mask, dtype=np.int32)
        rc = lib.orc_fix_set_atoms(self.h, atoms.n, _d(x), _d(v), _i(t), _i(m), groupbit)
        if rc:
            raise RuntimeError(f"orc_fix_set_atoms failed ({rc})")
        fdm = lib.orc_fix_fdm(self.h)
        self.ncells = lib.orc_fdm_ncells(fdm)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_fix_free(self.h)
            self.h = None

    def set_fext(self, fext):
        a = None if fext is None else np.ascontiguousarray(fext, dtype=np.float64)
        self.lib.orc_fix_set_fext(self.h, _d(a))

    def step(self, xi=None):
        a = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        rc = self.lib.orc_fix_step(self.h, _d(a))
        if rc:
            raise RuntimeError(f"orc_fix_step failed ({rc})")

    def get(self, what):
        sizes = {"x": 3, "v": 3, "f": 3, "f_eph": 3, "f_rng": 3, "w": 3, "xi": 3, "rho": 1, "alpha": 1, "array": 8}
        if what == "vector":
            out = np.zeros(2)
        elif what == "T":
            out = np.zeros(self.ncells)
        else:
            k = sizes[what]
            out = np.zeros((self.n, k) if k > 1 else self.n)
        rc = self.lib.orc_fix_get(self.h, what.encode(), _d(out))
        if rc:
            raise KeyError(what)
        return out

    def set(self, what, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if self.lib.orc_fix_set(self.h, what.encode(), _d(a)):
            raise KeyError(what)

    def neighbours(self, maxn=256):
        num = np.zeros(self.n, dtype=np.int32)
        own = np.full((self.n, maxn), -1, dtype=np.int32)
        self.lib.orc_fix_neigh(self.h, _i(num), _i(own), maxn)
        return num, own

    @property
    def nbuild(self):
        return self.lib.orc_fix_nbuild(self.h)

    def seconds(self, which=0):
        return self.lib.orc_fix_seconds(self.h, which)


_ref = None


def ref_available():
    return os.path.exists(REF_SO)


def reference_tree():
    """The reference tree _ref/libephref.so was compiled from (recorded by the
    Makefile in _ref/tree.txt), or EPH_REFERENCE_TREE; None when neither names
    an existing directory."""
    tree = os.environ.get("EPH_REFERENCE_TREE")
    rec = os.path.join(HERE, "_ref", "tree.txt")
    if not tree and os.path.exists(rec):
        tree = open(rec).read().strip()
    return tree if tree and os.path.isdir(tree) else None


def ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_SO)
        lib.ref_create.restype = C.c_void_p
        lib.ref_create.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_int, _dp, _dp, _ip, _ip, C.c_int, _dp, _dp,
                                   _dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_char_p, C.c_int]
        lib.ref_destroy.argtypes = [C.c_void_p]
        lib.ref_set_fext.argtypes = [C.c_void_p, _dp]
        lib.ref_step.argtypes = [C.c_void_p, _dp, C.c_long, C.c_char_p, C.c_int]
        lib.ref_get.argtypes = [C.c_void_p, C.c_char_p, _dp]
        lib.ref_get_T.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        lib.ref_get_neigh.argtypes = [C.c_void_p, _ip, _ip, C.c_int]
        lib.ref_nbuild.restype = C.c_long
        lib.ref_nbuild.argtypes = [C.c_void_p]
        lib.ref_save_temperature.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        lib.ref_save_state.argtypes = [C.c_void_p, C.c_char_p]
        _ref = lib
    return _ref


class RefFix:
    """The reference fix_eph.cpp, compiled unchanged, inside the engine
    stand-in."""

    def __init__(self, words, atoms, dt, skin=1.0, boltz=8.617343e-5, ftm2v=1.0 / 1.0364269e-4):
        lib = ref_lib()
        self.lib = lib
        err = C.create_string_buffer(512)
        mass = np.ascontiguousarray(atoms.mass, dtype=np.float64)
        x = np.ascontiguousarray(atoms.x, dtype=np.float64)
        v = np.ascontiguousarray(atoms.v, dtype=np.float64)
        t = np.ascontiguousarray(atoms.type, dtype=np.int32)
        m = np.ascontiguousarray(atoms.mask, dtype=np.int32)
        self.h = lib.ref_create(len(words), _argv(words), atoms.n, _d(x), _d(v), _i(t), _i(m), len(mass) - 1,
                                _d(mass), _d(atoms.boxlo), _d(atoms.boxhi), dt, boltz, ftm2v, skin, err, 512)
        if not self.h:
            raise RuntimeError(err.value.decode())
        self.n = atoms.n

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def set_fext(self, fext):
        a = None if fext is None else np.ascontiguousarray(fext, dtype=np.float64)
        self.lib.ref_set_fext(self.h, _d(a))

    def step(self, xi=None):
        a = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        err = C.create_string_buffer(512)
        rc = self.lib.ref_step(self.h, _d(a), 0 if a is None else a.size, err, 512)
        if rc:
            raise RuntimeError(err.value.decode())

    def get(self, what):
        sizes = {"x": 3, "v": 3, "f": 3, "f_eph": 3, "f_rng": 3, "w": 3, "xi": 3, "rho": 1, "array": 8}
        if what == "vector":
            out = np.zeros(2)
        else:
            k = sizes[what]
            out = np.zeros((self.n, k) if k > 1 else self.n)
        if self.lib.ref_get(self.h, what.encode(), _d(out)):
            raise KeyError(what)
        return out

    def get_T(self, grid, boxlo, boxhi):
        out = np.zeros(int(np.prod(grid)))
        lo = np.ascontiguousarray(boxlo, dtype=np.float64)
        hi = np.ascontiguousarray(boxhi, dtype=np.float64)
        self.lib.ref_get_T(self.h, grid[0], grid[1], grid[2], _d(lo), _d(hi), _d(out))
        return out

    def neighbours(self, maxn=256):
        num = np.zeros(self.n, dtype=np.int32)
        own = np.full((self.n, maxn), -1, dtype=np.int32)
        self.lib.ref_get_neigh(self.h, _i(num), _i(own), maxn)
        return num, own

    @property
    def nbuild(self):
        return self.lib.ref_nbuild(self.h)

    def save_temperature(self, path, n):
        self.lib.ref_save_temperature(self.h, path.encode(), n)

    def save_state(self, path):
        self.lib.ref_save_state(self.h, path.encode())


class RefBeta:
    """The reference EPH_Beta of a beta file (eph_beta.h), compiled unchanged."""

    def __init__(self, path):
        lib = ref_lib()
        lib.refb_load.restype = C.c_void_p
        lib.refb_load.argtypes = [C.c_char_p]
        lib.refb_free.argtypes = [C.c_void_p]
        lib.refb_eval.restype = C.c_double
        lib.refb_eval.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
        lib.refb_table.restype = C.c_long
        lib.refb_table.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        lib.refb_rho_cutoff.restype = C.c_double
        lib.refb_rho_cutoff.argtypes = [C.c_void_p]
        lib.refb_r_cutoff.restype = C.c_double
        lib.refb_r_cutoff.argtypes = [C.c_void_p]
        self.lib = lib
        self.h = lib.refb_load(path.encode())
        self.r_cutoff = lib.refb_r_cutoff(self.h)
        self.rho_cutoff = lib.refb_rho_cutoff(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.refb_free(self.h)
            self.h = None

    def eval(self, which, elem, xs):
        return np.array([self.lib.refb_eval(self.h, which, elem, float(x)) for x in np.atleast_1d(xs)])

    def table(self, which, elem):
        n = self.lib.refb_table(self.h, which, elem, None)
        out = np.zeros((n, 4))
        self.lib.refb_table(self.h, which, elem, _d(out))
        return out


class RefGrid:
    """The reference EPH_FDM (eph_fdm.h), compiled unchanged (one rank)."""

    def __init__(self, path=None, n=None, lo=None, hi=None, T=300.0, Ce=3.5e-6, rho=1.0, kappa=0.1):
        lib = ref_lib()
        lib.refg_create.restype = C.c_void_p
        lib.refg_create.argtypes = [C.c_long] * 3 + [_dp, _dp] + [C.c_double] * 4
        lib.refg_load.restype = C.c_void_p
        lib.refg_load.argtypes = [C.c_char_p]
        lib.refg_free.argtypes = [C.c_void_p]
        lib.refg_set_dt.argtypes = [C.c_void_p, C.c_double]
        lib.refg_insert_energy.argtypes = [C.c_void_p] + [C.c_double] * 4
        lib.refg_get_T.restype = C.c_double
        lib.refg_get_T.argtypes = [C.c_void_p] + [C.c_double] * 3
        lib.refg_get_T_total.restype = C.c_double
        lib.refg_get_T_total.argtypes = [C.c_void_p]
        lib.refg_solve.argtypes = [C.c_void_p]
        lib.refg_save_state.argtypes = [C.c_void_p, C.c_char_p]
        lib.refg_save_temperature.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        self.lib = lib
        if path is not None:
            self.h = lib.refg_load(path.encode())
        else:
            lo = np.ascontiguousarray(lo, dtype=np.float64)
            hi = np.ascontiguousarray(hi, dtype=np.float64)
            self.h = lib.refg_create(n[0], n[1], n[2], _d(lo), _d(hi), T, Ce, rho, kappa)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.refg_free(self.h)
            self.h = None

    def __getattr__(self, name):
        fn = getattr(self.lib, "refg_" + name)
        return lambda *a: fn(self.h, *[x.encode() if isinstance(x, str) else x for x in a])


GB_SO = os.path.join(HERE, "libgbfix.so")


def gb_available():
    return os.path.exists(GB_SO)


class GbFix:
    """The GB300 fix eph/gb (user-eph_gb300/lammps/fix_eph_gb.cpp) inside the
    engine stand-in, driven exactly like RefFix drives the reference fix."""

    _lib = None

    def __init__(self, words, atoms, dt, rc, mode=0, xi_host=1, skin=1.0, boltz=8.617343e-5,
                 ftm2v=1.0 / 1.0364269e-4):
        if GbFix._lib is None:
            lib = C.CDLL(GB_SO)
            lib.gbh_create.restype = C.c_void_p
            lib.gbh_create.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_int, _dp, _dp, _ip, _ip, C.c_int, _dp,
                                       _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_int, C.c_int, C.c_char_p, C.c_int]
            lib.gbh_destroy.argtypes = [C.c_void_p]
            lib.gbh_step.argtypes = [C.c_void_p, _dp, C.c_long, C.c_char_p, C.c_int]
            lib.gbh_get.argtypes = [C.c_void_p, C.c_char_p, _dp]
            lib.gbh_post_run.argtypes = [C.c_void_p]
            lib.gbh_modify.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
            GbFix._lib = lib
        lib = GbFix._lib
        self.lib = lib
        err = C.create_string_buffer(512)
        mass = np.ascontiguousarray(atoms.mass, dtype=np.float64)
        x = np.ascontiguousarray(atoms.x, dtype=np.float64)
        v = np.ascontiguousarray(atoms.v, dtype=np.float64)
        t = np.ascontiguousarray(atoms.type, dtype=np.int32)
        m = np.ascontiguousarray(atoms.mask, dtype=np.int32)
        self.h = lib.gbh_create(len(words), _argv(words), atoms.n, _d(x), _d(v), _i(t), _i(m), len(mass) - 1,
                                _d(mass), _d(atoms.boxlo), _d(atoms.boxhi), dt, boltz, ftm2v, skin, rc, mode,
                                xi_host, err, 512)
        if not self.h:
            raise RuntimeError(err.value.decode())
        self.n = atoms.n

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.gbh_destroy(self.h)
            self.h = None

    def step(self, xi=None):
        a = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        err = C.create_string_buffer(512)
        if self.lib.gbh_step(self.h, _d(a), 0 if a is None else a.size, err, 512):
            raise RuntimeError(err.value.decode())

    def modify(self, key, value):
        """fix_modify ID key value"""
        err = C.create_string_buffer(512)
        rc = self.lib.gbh_modify(self.h, key.encode(), str(value).encode(), err, 512)
        if rc:
            raise RuntimeError(f"fix_modify {key} {value}: {err.value.decode()} ({rc})")

    def get(self, what):
        k = {"x": 3, "v": 3, "f": 3, "array": 8}.get(what)
        out = np.zeros(2) if what == "vector" else np.zeros((self.n, k))
        if self.lib.gbh_get(self.h, what.encode(), _d(out)):
            raise KeyError(what)
        return out
