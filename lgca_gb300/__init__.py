"""GB300-native lattice-gas cellular automaton engine.

The compute path is liblgca_gpu.so (CUDA kernels for sm_103a behind the C ABI
declared in include/lgca_gpu.h).  This module binds that library with ctypes
and offers `GpuLattice`, a thin handle wrapper with numpy in/out used by the
tests, the benchmark and Python callers.  There is no CPU fallback: without
the library (or without a GPU) every call raises.

States exchanged with the host use the reference's format (keva92/lgca
src/lgca_bitset.h): a uint8 array of shape (dim_y, dim_x), bit d = channel d.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

HPP, FHP_I, FHP_II, FHP_III = 0, 1, 2, 3
FLUID, SOLID_NO_SLIP, SOLID_SLIP = 0, 1, 2
SHAPE_RECT, SHAPE_DISC, SHAPE_DISC_FLOAT = 0, 1, 2
NUM_DIR = {HPP: 4, FHP_I: 6, FHP_II: 7, FHP_III: 7}
MODEL_NAMES = {"HPP": HPP, "FHP_I": FHP_I, "FHP_II": FHP_II, "FHP_III": FHP_III}

LIB_PATH = _build.LIB

_lib = None


class LgcaError(RuntimeError):
    """A C-ABI call returned a non-zero lgca_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


def build(force: bool = False) -> str:
    return _build.build(force=force)


def lib() -> C.CDLL:
    """The loaded liblgca_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: run lgca_gb300.build() (nvcc, sm_103a) first")
        L = C.CDLL(LIB_PATH)
        vp, u64, i32p = C.c_void_p, C.c_uint64, C.POINTER(C.c_int32)
        sig = {
            "lgca_abi_version": (C.c_int, []),
            "lgca_status_string": (C.c_char_p, [C.c_int]),
            "lgca_last_error": (C.c_char_p, [vp]),
            "lgca_create": (C.c_int, [C.c_int, C.c_int, C.c_int, u64, C.POINTER(vp)]),
            "lgca_destroy": (C.c_int, [vp]),
            "lgca_info": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(u64), C.POINTER(u64)]),
            "lgca_set_step": (C.c_int, [vp, u64]),
            "lgca_trim_memory": (C.c_int, [C.c_int, u64]),
            "lgca_set_cell_types": (C.c_int, [vp, vp]),
            "lgca_get_cell_types": (C.c_int, [vp, vp]),
            "lgca_paint_cells": (C.c_int, [vp, C.c_int, C.c_int32, C.c_int64, C.c_int64,
                                           C.c_int64, C.c_int64]),
            "lgca_upload_state": (C.c_int, [vp, vp]),
            "lgca_download_state": (C.c_int, [vp, vp]),
            "lgca_download_state_async": (C.c_int, [vp, vp]),
            "lgca_init_random": (C.c_int, [vp, C.c_double, C.c_double]),
            "lgca_init_zero": (C.c_int, [vp]),
            "lgca_set_forcing_column": (C.c_int, [vp, C.c_int, C.c_double]),
            "lgca_set_chirality": (C.c_int, [vp, vp]),
            "lgca_set_temporal_depth": (C.c_int, [vp, C.c_int]),
            "lgca_set_kernel_variant": (C.c_int, [vp, C.c_int]),
            "lgca_step_plan": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
            "lgca_plan_shape": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int)]),
            "lgca_run_job_async": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, vp, vp, vp]),
            "lgca_collide_and_propagate_sums": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, vp]),
            "lgca_set_block_warps": (C.c_int, [vp, C.c_int]),
            "lgca_collide_and_propagate": (C.c_int, [vp, C.c_int]),
            "lgca_apply_body_force": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(u64)]),
            "lgca_count_particles": (C.c_int, [vp, C.POINTER(u64)]),
            "lgca_mean_velocity": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "lgca_block_sums": (C.c_int, [vp, C.c_int, vp, vp, vp]),
            "lgca_block_sums_device": (C.c_int, [vp, C.c_int, vp, vp, vp]),
            "lgca_block_sums_async": (C.c_int, [vp, C.c_int, vp, vp, vp]),
            "lgca_post_process": (C.c_int, [vp, C.c_int, vp, vp, vp, vp]),
            "lgca_sync": (C.c_int, [vp]),
            "lgca_clear_error": (C.c_int, [vp]),
            "lgca_set_wait_limit": (C.c_int, [vp, u64]),
            "lgca_test_withhold_progress": (C.c_int, [vp, C.c_int]),
            "lgca_stream": (vp, [vp]),
            "lgca_set_stream": (C.c_int, [vp, vp]),
            "lgca_state_device": (C.c_int, [vp, C.POINTER(vp), C.POINTER(C.c_size_t),
                                            C.POINTER(C.c_int)]),
            "lgca_device_bytes": (C.c_int, [vp, C.POINTER(C.c_size_t)]),
            "lgca_checkpoint_size": (C.c_int, [vp, C.POINTER(C.c_size_t)]),
            "lgca_checkpoint_save": (C.c_int, [vp, vp, C.c_size_t]),
            "lgca_checkpoint_load": (C.c_int, [vp, vp, C.c_size_t]),
            "lgca_batch_create": (C.c_int, [C.POINTER(vp)]),
            "lgca_batch_destroy": (C.c_int, [vp]),
            "lgca_batch_add": (C.c_int, [vp, vp]),
            "lgca_batch_remove": (C.c_int, [vp, vp]),
            "lgca_batch_size": (C.c_int, [vp, C.POINTER(C.c_int)]),
            "lgca_batch_step": (C.c_int, [vp, C.c_int]),
            "lgca_batch_step_each": (C.c_int, [vp, vp]),
            "lgca_batch_set_graph_steps": (C.c_int, [vp, C.c_int]),
            "lgca_batch_set_warp_tasks": (C.c_int, [vp, C.c_int]),
            "lgca_batch_sync": (C.c_int, [vp]),
            "lgca_batch_set_persistent": (C.c_int, [vp, C.c_int]),
            "lgca_batch_last_error": (C.c_char_p, [vp]),
            "lgca_batch_stream": (vp, [vp]),
            "lgca_apply_body_force_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, C.c_size_t,
                                                        C.c_int, vp, vp, u64, u64, C.c_int,
                                                        C.c_int, vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a) -> C.c_void_p | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(int(a))


def _check(h, status: int) -> None:
    if status != 0:
        msg = lib().lgca_last_error(h).decode(errors="replace")
        raise LgcaError(status, msg)


def trim_memory(device: int = 0, keep_bytes: int = 0) -> None:
    """Return the lattice memory pool's unused blocks beyond keep_bytes."""
    _check(None, lib().lgca_trim_memory(int(device), int(keep_bytes)))


def plan_shape(model: int, dim_x: int, dim_y: int, nsteps: int) -> tuple[int, int]:
    """GpuLattice.step_plan of a new lattice of this model and shape (default
    settings, current device), without creating it."""
    fam, n = C.c_int(), C.c_int()
    _check(None, lib().lgca_plan_shape(int(model), int(dim_x), int(dim_y), int(nsteps),
                                       C.byref(fam), C.byref(n)))
    return fam.value, n.value


class GpuLattice:
    """One lattice resident on the GPU, driven through the C ABI."""

    def __init__(self, model: int, dim_x: int, dim_y: int, seed: int = 0):
        h = C.c_void_p()
        st = lib().lgca_create(int(model), int(dim_x), int(dim_y), int(seed), C.byref(h))
        if st != 0:
            raise LgcaError(st, lib().lgca_last_error(None).decode(errors="replace"))
        self._h = h
        self.model, self.dim_x, self.dim_y, self.seed = int(model), int(dim_x), int(dim_y), int(seed)

    # lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            b = getattr(self, "_batch", None)
            if b is not None and self in b.members:  # keep the batch's member order in step
                b.members.remove(self)
            lib().lgca_destroy(self._h)  # also leaves its batch on the device side
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def shape(self):
        return (self.dim_y, self.dim_x)

    # configuration
    def set_cell_types(self, types: np.ndarray) -> None:
        t = np.ascontiguousarray(types, dtype=np.int32)
        assert t.shape == self.shape, (t.shape, self.shape)
        _check(self._h, lib().lgca_set_cell_types(self._h, _ptr(t)))

    def get_cell_types(self) -> np.ndarray:
        t = np.empty(self.shape, np.int32)
        _check(self._h, lib().lgca_get_cell_types(self._h, _ptr(t)))
        return t

    def paint_cells(self, shape: int, cell_type: int, a: int, b: int, c: int = 0,
                    d: int = 0) -> None:
        """Set the cells of a shape to one type on the device (see
        lgca_paint_cells): rectangle [a, c) x [b, d), integer disc centre
        (a, b) radius c, or the reference's float disc of diameter c."""
        _check(self._h, lib().lgca_paint_cells(self._h, int(shape), int(cell_type), int(a), int(b),
                                               int(c), int(d)))

    # the reference's geometry setters (src/lattice.cpp:222-335), painted on the device
    def apply_bc_periodic(self) -> None:
        self.paint_cells(SHAPE_RECT, FLUID, 0, 0, self.dim_x, self.dim_y)

    def apply_bc_pipe(self) -> None:
        W, H = self.dim_x, self.dim_y
        self.apply_bc_periodic()
        self.paint_cells(SHAPE_RECT, SOLID_NO_SLIP, 0, H - 1, W, H)  # north
        self.paint_cells(SHAPE_RECT, SOLID_NO_SLIP, 0, 0, W, 1)  # south

    def apply_bc_karman_vortex_street(self) -> None:
        self.apply_bc_pipe()
        self.paint_cells(SHAPE_DISC_FLOAT, SOLID_NO_SLIP, self.dim_x // 6, self.dim_y // 2,
                         self.dim_y // 3)

    def apply_bc_reflecting(self, bounce_type: str) -> None:
        if bounce_type not in ("back", "forward"):
            raise ValueError(f"invalid bounce type {bounce_type!r}")
        ct = SOLID_NO_SLIP if bounce_type == "back" else SOLID_SLIP
        W, H = self.dim_x, self.dim_y
        self.apply_bc_periodic()
        self.paint_cells(SHAPE_RECT, ct, W - 1, 0, W, H)  # east
        self.paint_cells(SHAPE_RECT, ct, 0, H - 1, W, H)  # north
        self.paint_cells(SHAPE_RECT, ct, 0, 0, 1, H)  # west
        self.paint_cells(SHAPE_RECT, ct, 0, 0, W, 1)  # south

    def upload(self, state: np.ndarray) -> None:
        s = np.ascontiguousarray(state, dtype=np.uint8)
        assert s.shape == self.shape
        _check(self._h, lib().lgca_upload_state(self._h, _ptr(s)))

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        s = np.empty(self.shape, np.uint8) if out is None else out
        _check(self._h, lib().lgca_download_state(self._h, _ptr(s)))
        return s

    def run_job_async(self, cells_in: np.ndarray | None, nsteps: int,
                      cells_out: np.ndarray | None, B: int = 0, sums: np.ndarray | None = None) -> None:
        """Upload cells_in (or keep the state), advance nsteps steps and queue
        the result into cells_out and, for B > 0, its B x B block sums into
        sums (int32, shape (3, ceil(H/B), ceil(W/B)): N, Jx2, Jy), all pinned
        for overlap and valid after sync(), in one call: where the resident
        kernel runs the steps, the layout conversions and the sums happen
        inside its launch."""
        for c in (cells_in, cells_out):
            assert c is None or (c.shape == self.shape and c.dtype == np.uint8 and
                                 c.flags.c_contiguous)
        n = jx = jy = None
        if B > 0:
            H, W = self.shape
            assert sums is not None and sums.dtype == np.int32 and sums.flags.c_contiguous
            assert sums.shape == (3, -(-H // B), -(-W // B))
            n, jx, jy = sums[0], sums[1], sums[2]
        _check(self._h, lib().lgca_run_job_async(self._h, _ptr(cells_in), int(nsteps),
                                                 _ptr(cells_out), int(B), _ptr(n), _ptr(jx),
                                                 _ptr(jy)))

    def collide_and_propagate_sums(self, nsteps: int, B: int, N_ptr: int, Jx2_ptr: int,
                                   Jy_ptr: int) -> None:
        """nsteps steps, then the B x B block sums of the result into device
        buffers (fused into the resident kernel's launch where it runs)."""
        _check(self._h, lib().lgca_collide_and_propagate_sums(self._h, int(nsteps), int(B),
                                                              _ptr(N_ptr), _ptr(Jx2_ptr),
                                                              _ptr(Jy_ptr)))

    def download_async(self, out: np.ndarray) -> None:
        """Queue a download into `out` (pinned for overlap); valid after sync()."""
        assert out.shape == self.shape and out.dtype == np.uint8 and out.flags.c_contiguous
        _check(self._h, lib().lgca_download_state_async(self._h, _ptr(out)))

    def init_random(self, p_move: float, p_rest: float | None = None) -> None:
        p_rest = p_move if p_rest is None else p_rest
        _check(self._h, lib().lgca_init_random(self._h, float(p_move), float(p_rest)))

    def init_zero(self) -> None:
        _check(self._h, lib().lgca_init_zero(self._h))

    def set_forcing_column(self, x: int, p: float) -> None:
        _check(self._h, lib().lgca_set_forcing_column(self._h, int(x), float(p)))

    def set_chirality(self, field: np.ndarray | None) -> None:
        f = None if field is None else np.ascontiguousarray(field, dtype=np.uint8)
        _check(self._h, lib().lgca_set_chirality(self._h, _ptr(f)))

    def set_temporal_depth(self, depth: int) -> None:
        _check(self._h, lib().lgca_set_temporal_depth(self._h, int(depth)))

    def set_block_warps(self, warps: int) -> None:
        """Warps per block of the one-step kernels (0 = chosen per launch)."""
        _check(self._h, lib().lgca_set_block_warps(self._h, int(warps)))

    def set_kernel_variant(self, variant: int) -> None:
        """0 auto, 1 one step per pass, 2 register wavefront, 3 shared-memory tiles,
        4 persistent bands, 5 one step per pass with two words per lane, 6 resident
        (state on chip across the steps of a call)."""
        _check(self._h, lib().lgca_set_kernel_variant(self._h, int(variant)))

    def step_plan(self, nsteps: int) -> tuple[int, int]:
        """(kernel family, step-kernel launches) of a call advancing nsteps
        steps: family 6 resident, 4 persistent bands, 1 passes."""
        fam, n = C.c_int(), C.c_int()
        _check(self._h, lib().lgca_step_plan(self._h, int(nsteps), C.byref(fam), C.byref(n)))
        return fam.value, n.value

    def set_step(self, t: int) -> None:
        _check(self._h, lib().lgca_set_step(self._h, int(t)))

    @property
    def step_count(self) -> int:
        t = C.c_uint64()
        _check(self._h, lib().lgca_info(self._h, None, None, None, None, C.byref(t)))
        return t.value

    # work
    def collide_and_propagate(self, nsteps: int = 1) -> None:
        _check(self._h, lib().lgca_collide_and_propagate(self._h, int(nsteps)))

    def apply_body_force(self, forcing: int, bf_dir: str | None = "x") -> int:
        n = C.c_uint64()
        d = ord(bf_dir) if bf_dir else 0
        _check(self._h, lib().lgca_apply_body_force(self._h, int(forcing), d, C.byref(n)))
        return n.value

    def count_particles(self) -> int:
        n = C.c_uint64()
        _check(self._h, lib().lgca_count_particles(self._h, C.byref(n)))
        return n.value

    def mean_velocity(self):
        ux, uy = C.c_float(), C.c_float()
        _check(self._h, lib().lgca_mean_velocity(self._h, C.byref(ux), C.byref(uy)))
        return ux.value, uy.value

    def block_sums(self, B: int):
        Hb, Wb = -(-self.dim_y // B), -(-self.dim_x // B)
        N = np.empty((Hb, Wb), np.int32)
        Jx2 = np.empty_like(N)
        Jy = np.empty_like(N)
        _check(self._h, lib().lgca_block_sums(self._h, int(B), _ptr(N), _ptr(Jx2), _ptr(Jy)))
        return N, Jx2, Jy

    def block_sums_async(self, B: int, N: np.ndarray, Jx2: np.ndarray, Jy: np.ndarray) -> None:
        """Enqueue block sums into host arrays (pinned for overlap); valid after sync()."""
        _check(self._h, lib().lgca_block_sums_async(self._h, int(B), _ptr(N), _ptr(Jx2), _ptr(Jy)))

    def block_sums_device(self, B: int, N_ptr: int, Jx2_ptr: int, Jy_ptr: int) -> None:
        _check(self._h, lib().lgca_block_sums_device(self._h, int(B), _ptr(N_ptr), _ptr(Jx2_ptr),
                                                     _ptr(Jy_ptr)))

    def post_process(self, r: int, cells: bool = True, means: bool = True):
        H, W = self.shape
        Hc, Wc = H // (2 * r), W // (2 * r)
        cd = np.empty((H, W), np.float32) if cells else None
        cm = np.empty((H, W, 2), np.float32) if cells else None
        md = np.empty((Hc, Wc), np.float32) if means else None
        mm = np.empty((Hc, Wc, 2), np.float32) if means else None
        _check(self._h, lib().lgca_post_process(self._h, int(r), _ptr(cd), _ptr(cm), _ptr(md),
                                                _ptr(mm)))
        return cd, cm, md, mm

    def sync(self) -> None:
        _check(self._h, lib().lgca_sync(self._h))

    def clear_error(self) -> None:
        """Acknowledge a persistent-kernel timeout (the state must then be reloaded)."""
        _check(self._h, lib().lgca_clear_error(self._h))

    def set_wait_limit(self, wait_ns: int) -> None:
        """Limit of one neighbour wait of the persistent kernel, in nanoseconds."""
        _check(self._h, lib().lgca_set_wait_limit(self._h, int(wait_ns)))

    def test_withhold_progress(self, block: int) -> None:
        """Test hook: block `block` of persistent launches never publishes its step."""
        _check(self._h, lib().lgca_test_withhold_progress(self._h, int(block)))

    def stream_ptr(self) -> int:
        return lib().lgca_stream(self._h) or 0

    def set_stream(self, stream_ptr: int | None) -> None:
        _check(self._h, lib().lgca_set_stream(self._h, _ptr(stream_ptr) if stream_ptr else None))

    def device_bytes(self) -> int:
        n = C.c_size_t()
        _check(self._h, lib().lgca_device_bytes(self._h, C.byref(n)))
        return n.value

    def checkpoint(self) -> bytes:
        n = C.c_size_t()
        _check(self._h, lib().lgca_checkpoint_size(self._h, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        _check(self._h, lib().lgca_checkpoint_save(self._h, _ptr(buf), n.value))
        return buf.tobytes()

    def restore(self, blob: bytes) -> None:
        buf = np.frombuffer(blob, np.uint8)
        _check(self._h, lib().lgca_checkpoint_load(self._h, _ptr(buf), buf.size))

    def state_device(self):
        p, ps, pitch = C.c_void_p(), C.c_size_t(), C.c_int()
        _check(self._h, lib().lgca_state_device(self._h, C.byref(p), C.byref(ps), C.byref(pitch)))
        return p.value, ps.value, pitch.value


class GpuBatch:
    """Many lattices advanced together (lgca_batch_*); members stay owned by
    the caller."""

    def __init__(self, graph_steps: int | None = None):
        h = C.c_void_p()
        st = lib().lgca_batch_create(C.byref(h))
        if st != 0:
            raise LgcaError(st, lib().lgca_batch_last_error(None).decode(errors="replace"))
        self._b = h
        self.members: list[GpuLattice] = []
        if graph_steps is not None:
            self._chk(lib().lgca_batch_set_graph_steps(self._b, int(graph_steps)))

    def _chk(self, st: int) -> None:
        if st != 0:
            raise LgcaError(st, lib().lgca_batch_last_error(self._b).decode(errors="replace"))

    def add(self, lattice: "GpuLattice") -> None:
        self._chk(lib().lgca_batch_add(self._b, lattice.handle))
        self.members.append(lattice)
        lattice._batch = self

    def remove(self, lattice: "GpuLattice") -> None:
        self._chk(lib().lgca_batch_remove(self._b, lattice.handle))
        self.members.remove(lattice)
        lattice._batch = None

    def step(self, nsteps: int) -> None:
        self._chk(lib().lgca_batch_step(self._b, int(nsteps)))

    def set_persistent(self, on: bool) -> None:
        """One cooperative launch per stretch of steps (grid barrier per step)."""
        self._chk(lib().lgca_batch_set_persistent(self._b, int(bool(on))))

    def set_warp_tasks(self, n: int) -> None:
        """Warp tasks per warp of the batched kernel (1, 2, 4 or 8; 0 = per call)."""
        self._chk(lib().lgca_batch_set_warp_tasks(self._b, int(n)))

    def step_each(self, nsteps) -> None:
        arr = np.ascontiguousarray(nsteps, dtype=np.int32)
        assert arr.size == len(self.members)
        self._chk(lib().lgca_batch_step_each(self._b, _ptr(arr)))

    def sync(self) -> None:
        self._chk(lib().lgca_batch_sync(self._b))

    def stream_ptr(self) -> int:
        return lib().lgca_batch_stream(self._b) or 0

    def close(self) -> None:
        if getattr(self, "_b", None):
            for m in self.members:
                m._batch = None
            lib().lgca_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


__all__ = ["GpuBatch", "GpuLattice", "LgcaError", "build", "lib", "plan_shape", "trim_memory",
           "HPP", "FHP_I", "FHP_II", "FHP_III",
           "FLUID", "SOLID_NO_SLIP", "SOLID_SLIP", "NUM_DIR"]
