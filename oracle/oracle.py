"""ctypes bindings of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries are wrapped:

* ``liblgca_oracle.so`` -- the plain-C restatement of the reference algorithm
  (oracle/lgca_oracle.c), built on every machine;
* ``_ref/libref_oracle.so`` -- the unmodified reference OMP_Lattice compiled
  with hooks (oracle/ref_harness.cpp); it only exists where the reference
  sources are present, and is used to pin the restatement.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module.  States are numpy uint8 arrays of shape (H, W), one byte
per cell with bit d = channel d (the reference's Bitset layout); cell types
are int32 arrays of the reference's CellType values.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liblgca_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_oracle.so")
# The reference checkout the harness is compiled from: $LGCA_REFERENCE_DIR, by
# default the path of the build machine's read-only copy.  The recipe names
# this path in this one place; the GPU machine has no copy and only uses the
# restatement and the committed fixtures.
REFERENCE_DIR = os.environ.get("LGCA_REFERENCE_DIR", "/root/reference")

HPP, FHP_I, FHP_II, FHP_III = 0, 1, 2, 3
FLUID, SOLID_NO_SLIP, SOLID_SLIP = 0, 1, 2
NUM_DIR = {HPP: 4, FHP_I: 6, FHP_II: 7, FHP_III: 7}

_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


class _Cfg(C.Structure):
    _fields_ = [
        ("model", C.c_int),
        ("W", C.c_int),
        ("H", C.c_int),
        ("seed", C.c_uint64),
        ("chir", C.c_void_p),
        ("force_x", C.c_int),
        ("force_thr", C.c_uint64),
    ]


def build(ref: bool = True) -> None:
    """Compile the restatement (and the reference harness when the reference
    sources are present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref and os.path.isdir(os.path.join(REFERENCE_DIR, "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_DIR}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        L.oracle_collide.restype = C.c_uint8
        L.oracle_collide.argtypes = [C.c_int, C.c_uint8, C.c_int]
        L.oracle_run.argtypes = [C.POINTER(_Cfg), C.c_void_p, _u8p, _u8p, C.c_uint64, C.c_int]
        L.oracle_init_bernoulli.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, _u8p,
                                            C.c_uint64, C.c_double, C.c_double]
        L.oracle_block_sums.argtypes = [C.c_int, C.c_int, C.c_int, _u8p, C.c_int, _i32p, _i32p, _i32p]
        L.oracle_cell_post_process.argtypes = [C.c_int, C.c_int, C.c_int, _u8p, _f32p, _f32p]
        L.oracle_mean_post_process.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p]
        L.oracle_count_particles.restype = C.c_uint64
        L.oracle_count_particles.argtypes = [C.c_int, C.c_int, _u8p]
        L.oracle_mean_velocity.argtypes = [C.c_int, C.c_int, C.c_void_p, _f32p, _f32p,
                                           C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.oracle_apply_body_force.restype = C.c_uint
        L.oracle_apply_body_force.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, _u8p,
                                              C.c_uint64, C.c_uint64, C.c_int, C.c_int]
        L.oracle_threads.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference harness not built (oracle/_ref/libref_oracle.so)")
        R = C.CDLL(REF_SO)
        R.ref_collide.restype = C.c_int
        R.ref_collide.argtypes = [C.c_int, C.c_int, C.c_int]
        R.ref_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, _u8p, C.c_uint64, C.c_int,
                              C.c_void_p, C.c_int, C.c_uint64, C.c_uint64, C.c_int]
        R.ref_post_process.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _u8p, _f32p, _f32p,
                                       _f32p, _f32p]
        R.ref_body_force.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, _u8p, C.c_uint64,
                                     C.c_uint64, C.c_int, C.c_int]
        R.ref_count_particles.restype = C.c_uint64
        R.ref_count_particles.argtypes = [C.c_int, C.c_int, C.c_int, _u8p]
        R.ref_mean_velocity.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, _u8p, _f32p]
        R.ref_dims.argtypes = [C.c_int, C.c_char_p, C.c_float, C.c_float, C.c_int,
                               np.ctypeslib.ndpointer(np.int32), _f32p]
        R.ref_geometry.argtypes = [C.c_int, C.c_int, C.c_int, C.c_char_p, _i32p]
        R.ref_init.argtypes = [C.c_int, C.c_int, C.c_int, C.c_char_p, _u8p]
        _ref = R
    return _ref


def prob_threshold(p: float) -> int:
    """floor(p * 2^32), clipped to [0, 2^32] (include/lgca/rng.h)."""
    if not p > 0.0:
        return 0
    if p >= 1.0:
        return 1 << 32
    return int(p * 4294967296.0)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _cfg(model, W, H, seed, chir=None, force_x=-1, force_p=0.0):
    return _Cfg(model, W, H, seed, _ptr(chir), force_x, prob_threshold(force_p))


# ---------------------------------------------------------------- restatement
def collide(model: int, state: int, p: int) -> int:
    return int(lib().oracle_collide(model, state, p))


def init_bernoulli(model, W, H, types=None, seed=1, p_move=0.2, p_rest=None):
    state = np.zeros((H, W), np.uint8)
    if p_rest is None:
        p_rest = p_move
    lib().oracle_init_bernoulli(model, W, H, _ptr(types), state, seed, p_move, p_rest)
    return state


def run(model, state, steps, types=None, seed=1, t0=0, chir=None, force_x=-1, force_p=0.0):
    """`steps` steps (forcing column, then pull+collide) from global step t0."""
    H, W = state.shape
    s = np.ascontiguousarray(state, np.uint8).copy()
    tmp = np.empty_like(s)
    cfg = _cfg(model, W, H, seed, chir, force_x, force_p)
    keep = (types, chir)
    lib().oracle_run(C.byref(cfg), _ptr(types), s, tmp, t0, steps)
    del keep
    return s


def block_sums(model, state, B):
    H, W = state.shape
    Hb, Wb = -(-H // B), -(-W // B)
    N = np.zeros((Hb, Wb), np.int32)
    Jx2 = np.zeros_like(N)
    Jy = np.zeros_like(N)
    lib().oracle_block_sums(model, W, H, np.ascontiguousarray(state), B, N, Jx2, Jy)
    return N, Jx2, Jy


def post_process(model, state, r):
    """(cell_density[H,W], cell_momentum[H,W,2], mean_density[Hc,Wc], mean_momentum[Hc,Wc,2])."""
    H, W = state.shape
    cd = np.zeros((H, W), np.float32)
    cm = np.zeros((H, W, 2), np.float32)
    Hc, Wc = H // (2 * r), W // (2 * r)
    md = np.zeros((Hc, Wc), np.float32)
    mm = np.zeros((Hc, Wc, 2), np.float32)
    L = lib()
    L.oracle_cell_post_process(model, W, H, np.ascontiguousarray(state), cd, cm)
    L.oracle_mean_post_process(W, H, r, cd, cm, md, mm)
    return cd, cm, md, mm


def count_particles(state) -> int:
    H, W = state.shape
    return int(lib().oracle_count_particles(W, H, np.ascontiguousarray(state)))


def mean_velocity(model, state, types=None):
    H, W = state.shape
    cd, cm, _, _ = post_process(model, state, 1)
    ux, uy = C.c_float(), C.c_float()
    lib().oracle_mean_velocity(W, H, _ptr(types), cd, cm, C.byref(ux), C.byref(uy))
    return ux.value, uy.value


def apply_body_force(model, state, forcing, types=None, seed=1, call=0, bf_dir="x"):
    H, W = state.shape
    s = np.ascontiguousarray(state, np.uint8).copy()
    bd = ord(bf_dir) if bf_dir else 0
    n = lib().oracle_apply_body_force(model, W, H, _ptr(types), s, seed, call, forcing, bd)
    return s, int(n)


# ---------------------------------------------------------------- reference
def ref_collide(model, state, p):
    return int(ref().ref_collide(model, state, p))


def ref_run(model, state, steps, types=None, seed=1, t0=0, chir=None, force_x=-1, force_p=0.0):
    H, W = state.shape
    s = np.ascontiguousarray(state, np.uint8).copy()
    mode = 1 if chir is not None else 0
    ref().ref_run(model, W, H, _ptr(types), s, seed, mode, _ptr(chir), force_x,
                  prob_threshold(force_p), t0, steps)
    return s


def ref_post_process(model, state, r):
    H, W = state.shape
    cd = np.zeros((H, W), np.float32)
    cm = np.zeros((H, W, 2), np.float32)
    Hc, Wc = H // (2 * r), W // (2 * r)
    md = np.zeros((Hc, Wc), np.float32)
    mm = np.zeros((Hc, Wc, 2), np.float32)
    ref().ref_post_process(model, W, H, r, np.ascontiguousarray(state), cd, cm, md, mm)
    return cd, cm, md, mm


def ref_apply_body_force(model, state, forcing, types=None, seed=1, call=0, bf_dir="x"):
    H, W = state.shape
    s = np.ascontiguousarray(state, np.uint8).copy()
    bd = ord(bf_dir) if bf_dir else 0
    ref().ref_body_force(model, W, H, _ptr(types), s, seed, call, forcing, bd)
    return s


def ref_count_particles(model, state):
    H, W = state.shape
    return int(ref().ref_count_particles(model, W, H, np.ascontiguousarray(state)))


def ref_mean_velocity(model, state, types=None):
    H, W = state.shape
    u = np.zeros(2, np.float32)
    ref().ref_mean_velocity(model, W, H, _ptr(types), np.ascontiguousarray(state), u)
    return float(u[0]), float(u[1])


def ref_dims(model, test_case, Re, Ma, r):
    oi = np.zeros(7, np.int32)
    of = np.zeros(3, np.float32)
    ref().ref_dims(model, test_case.encode(), Re, Ma, r, oi, of)
    return {"dim_x": int(oi[0]), "dim_y": int(oi[1]), "coarse_dim_x": int(oi[2]),
            "coarse_dim_y": int(oi[3]), "initial_forcing": int(oi[4]),
            "equilibrium_forcing": int(oi[5]), "bf_dir": int(oi[6]),
            "nu_s": float(of[0]), "c_s": float(of[1]), "u": float(of[2])}


def ref_geometry(model, W, H, bc):
    t = np.zeros((H, W), np.int32)
    rc = ref().ref_geometry(model, W, H, bc.encode(), t)
    if rc != 0:
        raise ValueError(bc)
    return t


def ref_init(model, W, H, what):
    s = np.zeros((H, W), np.uint8)
    if ref().ref_init(model, W, H, what.encode(), s) != 0:
        raise ValueError(what)
    return s
