"""Cell-type maps (int32, shape (dim_y, dim_x), values FLUID / SOLID_NO_SLIP /
SOLID_SLIP) for the reference's geometry setters and for the benchmark
workloads.  The maps are built on the host, as the reference builds
m_cell_type_cpu on the host, and handed to the GPU with set_cell_types.
"""
from __future__ import annotations

import numpy as np

FLUID, SOLID_NO_SLIP, SOLID_SLIP = 0, 1, 2


def periodic(W: int, H: int) -> np.ndarray:
    """Lattice::apply_bc_periodic (src/lattice.cpp:221-229): all FLUID."""
    return np.zeros((H, W), np.int32)


def pipe(W: int, H: int) -> np.ndarray:
    """Lattice::apply_bc_pipe (src/lattice.cpp:233-248): FLUID with the first
    and last rows SOLID_NO_SLIP (south = row 0, north = row H-1)."""
    t = periodic(W, H)
    t[0, :] = SOLID_NO_SLIP
    t[H - 1, :] = SOLID_NO_SLIP
    return t


def reflecting(W: int, H: int, bounce_type: str) -> np.ndarray:
    """Lattice::apply_bc_reflecting (src/lattice.cpp:311-334): all four edges
    SOLID_NO_SLIP ("back") or SOLID_SLIP ("forward")."""
    if bounce_type == "back":
        ct = SOLID_NO_SLIP
    elif bounce_type == "forward":
        ct = SOLID_SLIP
    else:
        raise ValueError(f"invalid bounce type {bounce_type!r}")
    t = periodic(W, H)
    t[:, W - 1] = ct
    t[H - 1, :] = ct
    t[:, 0] = ct
    t[0, :] = ct
    return t


def karman_reference(W: int, H: int) -> np.ndarray:
    """Lattice::apply_bc_karman_vortex_street (src/lattice.cpp:252-280): pipe
    walls plus a SOLID_NO_SLIP disc at (W/6, H/2) of diameter H/3 (integer
    divisions), tested as float(sqrt(dx^2 + dy^2)) < diameter / 2.0."""
    t = pipe(W, H)
    cx = W // 6
    cy = H // 2  # H/2 + 1/10*H with integer 1/10 = 0
    diameter = np.float32(H // 3)
    y, x = np.mgrid[0:H, 0:W]
    dist = np.sqrt((x - cx).astype(np.float64) ** 2 + (y - cy).astype(np.float64) ** 2)
    dist = dist.astype(np.float32).astype(np.float64)
    t[dist < np.float64(diameter) / 2.0] = SOLID_NO_SLIP
    return t


def disc(W: int, H: int, cx: int, cy: int, r: int, walls: bool = True) -> np.ndarray:
    """Disc obstacle: SOLID_NO_SLIP where (x-cx)^2 + (y-cy)^2 < r^2 (integer
    arithmetic), optionally inside pipe walls."""
    t = pipe(W, H) if walls else periodic(W, H)
    y, x = np.mgrid[0:H, 0:W]
    t[(x - cx) ** 2 + (y - cy) ** 2 < r * r] = SOLID_NO_SLIP
    return t
