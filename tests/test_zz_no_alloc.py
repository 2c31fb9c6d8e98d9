"""The allocation-free body force (lgca_apply_body_force_noalloc), called
through the C ABI on device buffers the caller owns, against the handle-based
entry point (lgca_apply_body_force) on the same lattice.

It serves callers that must not allocate device memory mid-run: a host that
has given its whole device budget to resident lattices, or one that cannot
accept the device-wide synchronisation of cudaMalloc/cudaFree between queued
steps.  Integer work: the comparison is bit-exact, on two calls in a row
(the second call reuses the shared scratch array the first one left behind).
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from lgca_gb300 import geometry as G

pytestmark = pytest.mark.gpu


def to_planes(state, D, pitch):
    """Reference byte format (H, W) -> D bit-planes (D, H, pitch) uint64."""
    H, W = state.shape
    out = np.zeros((D, H, pitch), np.uint64)
    x = np.arange(W)
    for d in range(D):
        bits = ((state >> d) & 1).astype(np.uint64) << (x % 64).astype(np.uint64)
        for w in range((W + 63) // 64):
            out[d, :, w] = np.bitwise_or.reduce(bits[:, 64 * w:64 * w + 64], axis=1)
    return out


def to_state(planes, W):
    D, H, _ = planes.shape
    s = np.zeros((H, W), np.uint8)
    x = np.arange(W)
    for d in range(D):
        words = planes[d][:, x // 64]
        s |= (((words >> (x % 64).astype(np.uint64)) & np.uint64(1)).astype(np.uint8) << d)
    return s


# (model, W, H, geometry, [(forcing, bf_dir) per call], device counter?)
CASES = [
    (3, 1000, 700, "karman", [(7000, "x"), (3000, "y")], True),
    (0, 640, 480, "pipe", [(5000, "x"), (2000, None)], False),
    (2, 333, 222, "disc", [(400, None), (900, "y")], True),
    # a lattice of exactly LGCA_NOALLOC_MAX_CELLS cells: the work arrays reach
    # the end of the fixed array, next to the count of the no-counter case
    (1, 2048, 1024, "pipe", [(20000, "x"), (20000, "y")], False),
    (3, 2048, 1024, "karman", [(30000, "y"), (10000, "x")], True),
]


def geometry(name, W, H):
    if name == "karman":
        return G.karman_reference(W, H)
    if name == "pipe":
        return G.pipe(W, H)
    return G.disc(W, H, W // 3, H // 2, H // 5)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"m{c[0]}_{c[1]}x{c[2]}_{c[3]}_{'dev' if c[5] else 'null'}")
def test_noalloc_body_force_equals_handle_path_on_two_calls(gpu, case):
    torch = pytest.importorskip("torch")
    model, W, H, geom, calls, counter = case
    seed = 6
    D = gpu.NUM_DIR[model]
    types = geometry(geom, W, H)

    # the existing entry point on a handle: two calls in a row
    with gpu.GpuLattice(model, W, H, seed=seed) as L:
        L.set_cell_types(types)
        L.init_random(0.3, 0.3)
        start = L.download()
        want = []
        for forcing, d in calls:
            n = L.apply_body_force(forcing, d)
            want.append((L.download(), n))

    # the allocation-free entry point on caller-owned device buffers
    pitch = ((W + 63) // 64 + 1) & ~1
    planes = torch.from_numpy(to_planes(start, D, pitch).view(np.int64)).cuda()
    solid = torch.from_numpy(to_planes((types == 1).astype(np.uint8), 1, pitch)[0].view(np.int64)).cuda()
    slip = torch.from_numpy(to_planes((types == 2).astype(np.uint8), 1, pitch)[0].view(np.int64)).cuda()
    rev = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    lib = gpu.lib()
    for call, ((forcing, d), (want_state, want_n)) in enumerate(zip(calls, want)):
        st = lib.lgca_apply_body_force_noalloc(model, W, H, planes.data_ptr(), H * pitch, pitch,
                                               solid.data_ptr(), slip.data_ptr(), seed, call,
                                               forcing, ord(d) if d else 0,
                                               rev.data_ptr() if counter else None,
                                               C.c_void_p(stream.cuda_stream))
        assert st == 0, lib.lgca_last_error(None)
        torch.cuda.synchronize()
        got = to_state(planes.cpu().numpy().view(np.uint64), W)
        assert np.array_equal(got, want_state), call
        if counter:
            assert int(rev.item()) == want_n


def test_noalloc_rejects_lattices_above_its_limit(gpu):
    lib = gpu.lib()
    W, H = 4096, 1024  # 4 Mi cells > LGCA_NOALLOC_MAX_CELLS (2 Mi)
    st = lib.lgca_apply_body_force_noalloc(3, W, H, C.c_void_p(16), H * 64, 64, None, None, 1, 0,
                                           10, ord("x"), None, None)
    assert st == 1
    assert b"limit" in lib.lgca_last_error(None)
