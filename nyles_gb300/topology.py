"""Subdomain topology: location, neighbours and array shapes.

Same functions and results as the reference's core/mpi/topology.py:29-157 and the
effective ``get_variable_shape`` (core/mpi/topology.py:253-300). This build runs one
subdomain per GPU, so only `procs = [1, 1, 1]` reaches the model, but the functions
keep their general behaviour.
"""
import itertools

POSSIBLE = ["closed", "perio_x", "perio_xy", "perio_y", "perio_xyz"]


def rank2loc(rank, procs):
    """(k, j, i) location of a rank in a grid of `procs` = [npz, npy, npx] subdomains."""
    return [rank // (procs[2] * procs[1]), (rank // procs[2]) % procs[1], rank % procs[2]]


def loc2rank(loc, procs):
    return (loc[0] * procs[1] + loc[1]) * procs[2] + loc[2]


def get_neighbours(location, procs, topology, incr=(1, 1, 1), extension=26):
    """Neighbour ranks keyed by direction (dk, dj, di); directions without a
    neighbour (closed walls) are absent."""
    if topology not in POSSIBLE:
        raise ValueError("unknown topology %r" % (topology,))
    if isinstance(location, int):
        k, j, i = rank2loc(location, procs)
    else:
        k, j, i = location
    nz, ny, nx = procs
    incz, incy, incx = incr
    sizes = {6: (1,), 18: (1, 2), 26: (1, 2, 3)}
    if extension not in sizes:
        raise ValueError("neighbours should be 6, 18 or 26")
    ngs = {}
    for dk, dj, di in itertools.product([-1, 0, 1], repeat=3):
        if abs(dk) + abs(dj) + abs(di) not in sizes[extension]:
            continue
        ok = True
        if "x" not in topology and not (0 <= i + di * incx < nx):
            ok = False
        if "y" not in topology and not (0 <= j + dj * incy < ny):
            ok = False
        if "z" not in topology and not (0 <= k + dk * incz < nz):
            ok = False
        if ok:
            loc = [(k + dk * incz) % nz, (j + dj * incy) % ny, (i + di * incx) % nx]
            ngs[(dk, dj, di)] = loc2rank(loc, procs)
    return ngs


def get_variable_shape(innersize, ngbs, nh):
    """Array extents and interior index ranges (k0, k1, j0, j1, i0, i1): a halo of nh
    on each side that has a neighbour, nothing otherwise."""
    size = list(innersize)
    starts, ends = [], []
    for axis, (lo, hi) in enumerate([((-1, 0, 0), (1, 0, 0)), ((0, -1, 0), (0, 1, 0)), ((0, 0, -1), (0, 0, 1))]):
        s0 = 0
        if lo in ngbs:
            size[axis] += nh
            s0 = nh
        e = size[axis]
        if hi in ngbs:
            size[axis] += nh
        starts.append(s0)
        ends.append(e)
    return size, (starts[0], ends[0], starts[1], ends[1], starts[2], ends[2])


def periodic_flags(topology):
    """(x, y, z) periodicity of a geometry name."""
    return ("x" in topology, "y" in topology, "z" in topology)
