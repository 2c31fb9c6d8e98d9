"""Lattice parameters and the small initialisers of the reference Lattice
class, restated on the host (numpy float32 mirrors the reference's
`Real = float`, src/lgca_common.h:46).  The C++ GB_Lattice wrapper
(include/lgca/gb_lattice.h) carries the same formulas."""
from __future__ import annotations

import math

import numpy as np

NUM_DIR = {0: 4, 1: 6, 2: 7, 3: 7}
INV_DIR0 = {0: 2, 1: 3, 2: 3, 3: 3}  # INV_DIR[0] of each model


def lattice_parameters(model: int, test_case: str, Re: float, Ma: float, r: int) -> dict:
    """Lattice<M>::Lattice (src/lattice.cpp:29-157) and the forcing amounts of
    get_initial_forcing / get_equilibrium_forcing (src/lattice.cpp:446-461)."""
    f32 = np.float32
    D = NUM_DIR[model]
    Re, Ma = f32(Re), f32(Ma)
    d = f32(f32(1.0) / f32(D))
    nu = f32(1.0 / 12.0 * 1.0 / (float(d) * math.pow(1.0 - float(d), 3.0)) - 1.0 / 8.0)
    g = f32(2 / (2 + 2.0) * (1.0 - 2.0 * float(d)) / (1.0 - float(d)))
    nu_s = f32(nu / g)
    c_s = f32(float(f32(1.0)) / math.sqrt(2))
    u = f32(Ma * c_s)
    if test_case == "pipe":
        dim_y = int(float(f32(f32(Re * nu_s) / u)) + 0.5)
    elif test_case == "karman":
        diameter = f32(f32(Re * nu_s) / u)
        dim_y = int(3.0 * float(diameter) + 0.5)
    elif test_case == "collision":
        dim_y = 8
    elif test_case in ("diffusion", "periodic", "box"):
        dim_y = int(Re)
    else:
        raise ValueError(f"invalid test case {test_case!r}")
    dim_y += 2 * r - (dim_y % (2 * r))
    dim_x = 2 * dim_y if test_case in ("pipe", "karman", "collision") else dim_y
    if test_case == "collision":
        dim_x += 1
    bf_dir = ord("x") if test_case in ("pipe", "karman") else 0
    cells = dim_x * dim_y
    forcing = f32((8.0 * float(nu_s) * float(Ma) * float(c_s)) / math.pow(float(f32(dim_y)), 2.0))
    return dict(dim_x=dim_x, dim_y=dim_y, coarse_dim_x=dim_x // (2 * r),
                coarse_dim_y=dim_y // (2 * r), initial_forcing=int(0.01 * cells),
                equilibrium_forcing=int(math.ceil(0.5 * cells * float(forcing))), bf_dir=bf_dir,
                nu_s=float(nu_s), c_s=float(c_s), u=float(u))


def init_single(W: int, H: int, occupied_nodes) -> np.ndarray:
    """Lattice::init_single (src/lattice.cpp:297-308): node n = channel n % 8
    of cell n // 8."""
    s = np.zeros(W * H, np.uint8)
    for n in occupied_nodes:
        s[n // 8] |= np.uint8(1 << (n % 8))
    return s.reshape(H, W)


def init_single_collision(model: int, W: int, H: int) -> np.ndarray:
    """Lattice::init_single_collision (src/lattice.cpp:283-294): one particle
    in channel 0 of cell W*H/2+1 and one in channel INV_DIR[0] of cell
    W*H/2+5."""
    c = W * H // 2
    return init_single(W, H, [(c + 1) * 8, (c + 5) * 8 + INV_DIR0[model]])
