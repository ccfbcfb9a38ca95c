"""Seeded synthetic cases in the reference's own input formats.

The reference reads a gmsh v2 ASCII mesh (``RootProcess::read``,
NS/RootStructure.cpp:428-487: it skips tokens up to ``$Nodes``, reads
``id x y z`` per node, two more tokens, then ``id type ntags tags... nodes...``
per element, node ids 1-based) and a comma-separated ``param.in``
(NS/readparamfile.cpp:10-344).  This module writes both for the workloads the
solver is measured on:

* ``cavity``  -- lid-driven cavity in the unit cube, n^3 hexahedra (gmsh type 5),
  walls (rid 1, ``Hwall``), lid z=1 (rid 2, ``inlet`` u=(1,0,0)), fluid rid 3.
  The lid is an inlet because the reference forces zero velocity on walls
  (NS/navier_bc.cpp:19-24).
* ``channel`` -- box [0,L]x[0,1]x[0,1] of nx*ny*nz hexes, each split into six
  Kuhn tetrahedra along the v0-v6 diagonal (conforming), interior nodes jittered
  by U(-j*h, j*h) per coordinate, boundary triangles taken from the tets'
  once-occurring faces; inlet x=0 (rid 1), outlet x=L (rid 2), walls (rid 3),
  fluid rid 4.

Coordinates are printed with ``%.17g`` so they round-trip bit-exactly.
"""
from __future__ import annotations

import os
import numpy as np

# Kuhn subdivision of a hex with gmsh local numbering
# v0=(0,0,0) v1=(1,0,0) v2=(1,1,0) v3=(0,1,0) v4=(0,0,1) v5=(1,0,1) v6=(1,1,1) v7=(0,1,1):
# one tet per axis permutation, path v0 -> +e_a -> +e_a+e_b -> v6.
_KUHN = np.array([
    [0, 1, 2, 6],   # x, y, z
    [0, 1, 5, 6],   # x, z, y
    [0, 3, 2, 6],   # y, x, z
    [0, 3, 7, 6],   # y, z, x
    [0, 4, 5, 6],   # z, x, y
    [0, 4, 7, 6],   # z, y, x
], dtype=np.int64)


def _grid_nodes(nx, ny, nz, lx, ly, lz):
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    zs = np.linspace(0.0, lz, nz + 1)
    z, y, x = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def _node_id(i, j, k, nx, ny):
    return i + (nx + 1) * (j + (ny + 1) * k)


def _hex_connectivity(nx, ny, nz):
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i = i.transpose(2, 1, 0).ravel()
    j = j.transpose(2, 1, 0).ravel()
    k = k.transpose(2, 1, 0).ravel()
    n = lambda a, b, c: _node_id(a, b, c, nx, ny)
    return np.stack([n(i, j, k), n(i + 1, j, k), n(i + 1, j + 1, k), n(i, j + 1, k),
                     n(i, j, k + 1), n(i + 1, j, k + 1), n(i + 1, j + 1, k + 1), n(i, j + 1, k + 1)],
                    axis=1).astype(np.int64)


def _jitter(nodes, nx, ny, nz, hx, hy, hz, amp, rng, planar):
    """Move interior nodes by U(-amp*h, amp*h) per coordinate.

    ``planar=True`` moves whole grid planes (x depends on i only, ...), which keeps
    every hex face planar: the reference rejects faces whose two-triangle area and
    vector area differ by more than 1e-4 (NS/geometry.cpp:604-610).
    """
    if amp <= 0.0:
        return nodes
    out = nodes.copy()
    if planar:
        dx = rng.uniform(-amp * hx, amp * hx, nx + 1); dx[0] = dx[-1] = 0.0
        dy = rng.uniform(-amp * hy, amp * hy, ny + 1); dy[0] = dy[-1] = 0.0
        dz = rng.uniform(-amp * hz, amp * hz, nz + 1); dz[0] = dz[-1] = 0.0
        ii = np.tile(np.arange(nx + 1), (ny + 1) * (nz + 1))
        jj = np.tile(np.repeat(np.arange(ny + 1), nx + 1), nz + 1)
        kk = np.repeat(np.arange(nz + 1), (nx + 1) * (ny + 1))
        out[:, 0] += dx[ii]
        out[:, 1] += dy[jj]
        out[:, 2] += dz[kk]
        return out
    ii = np.tile(np.arange(nx + 1), (ny + 1) * (nz + 1))
    jj = np.tile(np.repeat(np.arange(ny + 1), nx + 1), nz + 1)
    kk = np.repeat(np.arange(nz + 1), (nx + 1) * (ny + 1))
    interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)
    d = rng.uniform(-1.0, 1.0, (nodes.shape[0], 3)) * amp * np.array([hx, hy, hz])
    out[interior] += d[interior]
    return out


def _write_gmsh(path, nodes, elems):
    """elems: list of (type, tags(M,2) int, conn(M,k) int 0-based)."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % nodes.shape[0])
        ids = np.arange(1, nodes.shape[0] + 1)
        np.savetxt(f, np.column_stack([ids, nodes]), fmt=["%d", "%.17g", "%.17g", "%.17g"])
        f.write("$EndNodes\n$Elements\n")
        total = sum(c.shape[0] for _, _, c in elems)
        f.write("%d\n" % total)
        eid = 1
        for etype, tags, conn in elems:
            m = conn.shape[0]
            cols = [np.arange(eid, eid + m), np.full(m, etype), np.full(m, 2), tags[:, 0], tags[:, 1]]
            cols += [conn[:, q] + 1 for q in range(conn.shape[1])]
            np.savetxt(f, np.column_stack(cols).astype(np.int64), fmt="%d")
            eid += m
        f.write("$EndElements\n")


def cavity_mesh(n, jitter=0.0, seed=0, planar=True):
    """n^3 hex cavity. Returns (nodes, elems) for ``_write_gmsh``."""
    h = 1.0 / n
    nodes = _grid_nodes(n, n, n, 1.0, 1.0, 1.0)
    rng = np.random.default_rng(seed)
    nodes = _jitter(nodes, n, n, n, h, h, h, jitter, rng, planar)
    hexes = _hex_connectivity(n, n, n)
    nid = lambda a, b, c: _node_id(a, b, c, n, n)
    quads, rids = [], []
    a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = a.ravel(); b = b.ravel()
    # x = 0 / x = 1 (walls)
    for i0, rid in ((0, 1), (n, 1)):
        quads.append(np.stack([nid(i0, a, b), nid(i0, a + 1, b), nid(i0, a + 1, b + 1), nid(i0, a, b + 1)], 1)); rids.append(np.full(a.size, rid))
    for j0, rid in ((0, 1), (n, 1)):
        quads.append(np.stack([nid(a, j0, b), nid(a + 1, j0, b), nid(a + 1, j0, b + 1), nid(a, j0, b + 1)], 1)); rids.append(np.full(a.size, rid))
    for k0, rid in ((0, 1), (n, 2)):
        quads.append(np.stack([nid(a, b, k0), nid(a + 1, b, k0), nid(a + 1, b + 1, k0), nid(a, b + 1, k0)], 1)); rids.append(np.full(a.size, rid))
    quads = np.concatenate(quads).astype(np.int64)
    rids = np.concatenate(rids).astype(np.int64)
    qt = np.stack([rids, rids], 1)
    ht = np.full((hexes.shape[0], 2), 3, dtype=np.int64)
    return nodes, [(3, qt, quads), (5, ht, hexes)]


def channel_mesh(nx, ny, nz, length=10.0, jitter=0.15, seed=2026):
    """Kuhn-tet channel. Returns (nodes, elems)."""
    hx, hy, hz = length / nx, 1.0 / ny, 1.0 / nz
    nodes = _grid_nodes(nx, ny, nz, length, 1.0, 1.0)
    rng = np.random.default_rng(seed)
    nodes = _jitter(nodes, nx, ny, nz, hx, hy, hz, jitter, rng, planar=False)
    hexes = _hex_connectivity(nx, ny, nz)
    tets = hexes[:, _KUHN].reshape(-1, 4)
    # faces of every tet: opposite-vertex triangles
    fidx = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
    faces = tets[:, fidx].reshape(-1, 3)
    key = np.sort(faces, axis=1)
    kview = key[:, 0] * (nodes.shape[0] ** 2) + key[:, 1] * nodes.shape[0] + key[:, 2]
    uniq, first, counts = np.unique(kview, return_index=True, return_counts=True)
    bfaces = faces[first[counts == 1]]
    # classify by which side of the (unjittered) box the face lies on
    ii = bfaces % (nx + 1)
    jj = (bfaces // (nx + 1)) % (ny + 1)
    kk = bfaces // ((nx + 1) * (ny + 1))
    rid = np.full(bfaces.shape[0], 3, dtype=np.int64)
    rid[np.all(ii == 0, axis=1)] = 1
    rid[np.all(ii == nx, axis=1)] = 2
    order = np.argsort(rid, kind="stable")
    bfaces, rid = bfaces[order], rid[order]
    tt = np.full((tets.shape[0], 2), 4, dtype=np.int64)
    return nodes, [(2, np.stack([rid, rid], 1), bfaces.astype(np.int64)), (4, tt, tets.astype(np.int64))]


def _time_and_physics(steps, residual, time, energy, density):
    """The time line (steady, or transient with (dt, total_time, MaxOuterStep, scheme)) and the
    optional energy / density lines of a param.in."""
    if time is None:
        lines = f"steady,{steps},{residual!r}\n"
    else:
        dt, total, outer, scheme = time
        lines = f"transient,{dt!r},{total!r},{outer},{scheme}\n"
    if energy:
        lines += "energy,on\n"
    if density:
        lines += f"density,{density}\n"
    return lines


def gas_density(T, p_ref=1.01325e5):
    """Perfect-gas density at gauge pressure 0 with the reference's constants (cp 1006, gamma 1.4)."""
    cp = 1006.
    cv = cp / 1.4
    return p_ref / ((cp - cv) * T)


def cavity_param(mesh_name, steps=200, mu=0.01, lid=1.0, residual=1e-300, time=None, energy=False, density=0,
                 wall_t=None, lid_t=300):
    ro = gas_density(300.0) if density == 1 else 1
    ro_lid = gas_density(lid_t) if density == 1 else 1
    wall = "bound,1,Hwall,walls,0\n" if wall_t is None else f"bound,1,Twall,walls,{wall_t!r}\n"
    return (f"gridfile,{mesh_name}\n"
            + _time_and_physics(steps, residual, time, energy, density) +
            "turbulence,no\n"
            "relaxation,0.6,0.5,0.8\n"
            f"initflow,0,0,0,{ro!r},300,{mu!r},0,0\n"
            + wall +
            f"bound,2,inlet,lid,{lid!r},0,0,0,{ro_lid!r},{lid_t!r},0,0\n"
            f"volumn,3,fluid,fluid,0,0,0,{ro!r},300,{mu!r},0,0\n"
            "output,100000,tecplot\n")


def channel_param(mesh_name, steps=500, u_in=1.0, mu=2e-5, residual=1e-300, time=None, energy=False,
                  wall_t=None, t_in=300):
    k = 1.5 * (0.05 * u_in) ** 2
    eps = 0.09 ** 0.75 * k ** 1.5 / 0.07
    wall = "bound,3,Hwall,walls,0\n" if wall_t is None else f"bound,3,Twall,walls,{wall_t!r}\n"
    return (f"gridfile,{mesh_name}\n"
            "turbulence,ke\n"
            + _time_and_physics(steps, residual, time, energy, 0) +
            "relaxation,0.6,0.5,0.8\n"
            f"initflow,{u_in!r},0,0,1,300,{mu!r},{k!r},{eps!r}\n"
            f"bound,1,inlet,inlet,{u_in!r},0,0,0,1,{t_in!r},{k!r},{eps!r}\n"
            "bound,2,outlet,outlet,0\n"
            + wall +
            f"volumn,4,fluid,fluid,{u_in!r},0,0,1,300,{mu!r},{k!r},{eps!r}\n"
            "output,100000,tecplot\n")


def write_case(directory, kind, **kw):
    """Write ``<directory>/case.msh`` + ``<directory>/param.in``; return the param path."""
    os.makedirs(directory, exist_ok=True)
    mesh = os.path.join(directory, "case.msh")
    if kind == "cavity":
        n = kw.pop("n")
        nodes, elems = cavity_mesh(n, jitter=kw.pop("jitter", 0.0), seed=kw.pop("seed", 0),
                                   planar=kw.pop("planar", True))
        text = cavity_param("case.msh", **kw)
    elif kind == "channel":
        nx, ny, nz = kw.pop("nx"), kw.pop("ny"), kw.pop("nz")
        nodes, elems = channel_mesh(nx, ny, nz, length=kw.pop("length", 10.0),
                                    jitter=kw.pop("jitter", 0.15), seed=kw.pop("seed", 2026))
        text = channel_param("case.msh", **kw)
    else:
        raise ValueError(kind)
    _write_gmsh(mesh, nodes, elems)
    param = os.path.join(directory, "param.in")
    with open(param, "w") as f:
        f.write(text)
    return param


def compress_msh(src, dst):
    """Writes the compressed binary form of a gmsh v2 ASCII file, line by line as the reference's
    converter does (postCycas.py:compressIn): nothing before ``$Nodes``; a line with one number
    becomes an int64 (the node and element counts); a node line becomes int32 id + three doubles;
    an element line becomes its numbers as int32; section markers are dropped.  The result is
    what ``Case(param, msh_binary=True)`` (RootProcess::readBin) reads."""
    import struct

    found_node = found_elem = False
    with open(src) as f, open(dst, "wb") as out:
        for line in f:
            if line.startswith("$Nodes"):
                found_node = True
                continue
            if line.startswith("$Elements"):
                found_elem = True
                continue
            if line.startswith("$EndNodes") or line.startswith("$EndElements"):
                continue
            nums = line.split()
            if not found_node or not nums:
                continue
            if len(nums) == 1:
                out.write(struct.pack("<q", int(nums[0])))
            elif found_elem:
                out.write(struct.pack("<%di" % len(nums), *[int(x) for x in nums]))
            else:
                out.write(struct.pack("<i3d", int(nums[0]), float(nums[1]), float(nums[2]), float(nums[3])))
