"""The argument behind the projection's fast paths, checked on the CPU.

A tile runs K red/black sweeps of apply_projection_at (src/fluid.cu:229-262)
on its region (owned cells plus a halo of 2K) and keeps only its owned faces.
Each half-sweep need only update the cells within `reach` (the half-sweeps
still to come) of the owned tile: the cone. The all-fluid loop and the flag
loop update cells off the cone too. That is harmless because the cone shrinks
by one cell per side each half-sweep, so whatever a cell off the cone writes
reaches only cells that are off the cone from then on. Here three tiles are
swept three ways - only the cone, every cell of the region, and every cell
with the cells off the cone writing random values - and the owned faces must
equal those of the same sweeps on the whole grid, exactly (float64, the same
operations in the same order for every cell that matters)."""
import numpy as np
import pytest


def make_grid(rng, W, H):
    solid = np.zeros((W, H), bool)
    solid[0, :] = solid[:, 0] = solid[:, H - 1] = True
    cx, cy, r = W * 0.45, H * 0.55, min(W, H) * 0.15
    xs, ys = np.meshgrid(np.arange(W), np.arange(H), indexing="ij")
    solid |= (xs - cx) ** 2 + (ys - cy) ** 2 < r * r
    solid |= rng.random((W, H)) < 0.03
    fluid = ~solid
    s = np.zeros((W, H))
    s[1:, :] += fluid[:-1, :]
    s[:-1, :] += fluid[1:, :]
    s[:, 1:] += fluid[:, :-1]
    s[:, :-1] += fluid[:, 1:]
    u = rng.standard_normal((W, H))
    v = rng.standard_normal((W, H))
    return solid, s, u, v


def half_sweep(u, v, solid, s, colour, o, cells, garbage=None):
    """apply_projection_at on `cells` (a list of (i, j) of one colour), in
    place; cells in `garbage` write a random velocity change instead."""
    for i, j in cells:
        if solid[i, j]:
            continue
        div = u[i + 1, j] - u[i, j] + v[i, j + 1] - v[i, j]
        vd = o * (div / s[i, j])
        if garbage is not None and (i, j) in garbage[0]:
            vd = garbage[1].standard_normal()
        if not solid[i - 1, j]:
            u[i, j] += vd
        if not solid[i + 1, j]:
            u[i + 1, j] -= vd
        if not solid[i, j - 1]:
            v[i, j] += vd
        if not solid[i, j + 1]:
            v[i, j + 1] -= vd


def grid_cells(W, H, colour):
    return [(i, j) for j in range(1, H - 1) for i in range(1, W - 1) if (i + j) % 2 == colour]


def tile_sweeps(u, v, solid, s, K, o, gx0, gy0, RW, RH, mode, rng):
    """K sweeps on the region [gx0, gx0 + RW) x [gy0, gy0 + RH), on copies."""
    u, v = u.copy(), v.copy()
    halo = 2 * K
    W, H = solid.shape
    for t in range(K):
        for colour in (0, 1):
            reach = 2 * (K - t) - 1 - colour
            lo = halo - 1 - reach
            inside, cone = [], set()
            for y in range(RH - 1):
                for x in range(RW - 1):
                    i, j = gx0 + x, gy0 + y
                    if not (0 < i < W - 1 and 0 < j < H - 1) or (i + j) % 2 != colour:
                        continue
                    in_cone = lo <= x < RW - halo + reach and lo <= y < RH - halo + reach
                    if in_cone:
                        cone.add((i, j))
                    if in_cone or mode != "cone":
                        inside.append((i, j))
            off = {c for c in inside if c not in cone}
            half_sweep(u, v, solid, s, colour, o, inside,
                       garbage=(off, rng) if mode == "garbage" else None)
    return u, v


@pytest.mark.parametrize("mode", ["cone", "all", "garbage"])
@pytest.mark.parametrize("tile", [(0, 0), (1, 1), (2, 1)])
def test_owned_faces_do_not_depend_on_cells_off_the_cone(mode, tile):
    rng = np.random.default_rng(11)
    W, H, K, o = 46, 38, 3, 1.9
    halo, TX, TY = 2 * K, 14, 12
    solid, s, u0, v0 = make_grid(rng, W, H)
    u, v = u0.copy(), v0.copy()
    for _ in range(K):
        for colour in (0, 1):
            half_sweep(u, v, solid, s, colour, o, grid_cells(W, H, colour))
    tx, ty = tile
    gx0, gy0 = tx * TX - halo, ty * TY - halo
    RW, RH = TX + 2 * halo, TY + 2 * halo
    # Region cells off the grid are never updated; the rest start from the
    # grid's values.
    ut, vt = tile_sweeps(u0, v0, solid, s, K, o, gx0, gy0, RW, RH, mode,
                         np.random.default_rng(5))
    ox0, oy0 = tx * TX, ty * TY
    ox1, oy1 = min(ox0 + TX, W), min(oy0 + TY, H)
    assert np.array_equal(ut[ox0:ox1, oy0:oy1], u[ox0:ox1, oy0:oy1])
    assert np.array_equal(vt[ox0:ox1, oy0:oy1], v[ox0:ox1, oy0:oy1])
    # ...and the check has teeth: the faces just outside the owned tile
    # (the halo) differ from the grid's once the region is swept.
    if mode == "garbage":
        assert not np.array_equal(ut, u)
