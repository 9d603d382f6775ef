"""Comparison of two solutions of the A-V system, block by block.

A solution is the reference's ``x_vec`` (3D/QMS_3D.f90:172-176): ``[Ax|Ay|Az|V]``
in Fortran order.  Three quantities are compared:

* **A**, the edge unknowns, directly;
* **V**, the nodal potential, after fixing its gauge.  A body of conductors that
  no conducting path links to the grounded (Dirichlet) shell has a potential
  pinned only through the 1e-12 S/m air floor (F:1236-1285): a mode ~19
  decades below the conductor scale, so every FP64 solver leaves an arbitrary
  constant on it.  V is compared on the conducting nodes (nodes with at least
  one conducting edge), with the mean over each floating body removed from
  both sides.  Potentials in air carry no current and are left out;
* **H** (B / mu at the cell centres, the field the reference dumps,
  F:1346-1376), from the cubes the caller passes.

Edge conductivities follow the reference: the mean of the four cells around
the edge (F:264-266), formed only for node indices 2..size (F:258-260).
"""
from __future__ import annotations

import numpy as np

SIGMA_CONDUCTING = 1.0     # S/m: edges above this carry current; the air floor is 1e-12


def _cell_sigma(inp, geom):
    xs, ys, zs = inp.xs, inp.ys, inp.zs
    g = np.asarray(geom).reshape((xs, ys, zs), order="F")
    sig = np.zeros((3, xs, ys, zs))
    for row in inp.props_table():
        m = g == row[0]
        for a in range(3):
            sig[a][m] = row[4 + a]
    return sig


def edge_sigma(inp, geom):
    """sigma on the x-, y- and z-edges: arrays (xs, Ny, Nz), (Nx, ys, Nz), (Nx, Ny, zs)."""
    xs, ys, zs = inp.xs, inp.ys, inp.zs
    sig = _cell_sigma(inp, geom)
    out = []
    for a in range(3):
        s = np.pad(sig[a], 1)                 # cells with a zero halo
        if a == 0:
            se = 0.25 * (s[1:-1, :-1, :-1] + s[1:-1, 1:, :-1] + s[1:-1, :-1, 1:] + s[1:-1, 1:, 1:])
        elif a == 1:
            se = 0.25 * (s[:-1, 1:-1, :-1] + s[1:, 1:-1, :-1] + s[:-1, 1:-1, 1:] + s[1:, 1:-1, 1:])
        else:
            se = 0.25 * (s[:-1, :-1, 1:-1] + s[1:, :-1, 1:-1] + s[:-1, 1:, 1:-1] + s[1:, 1:, 1:-1])
        # the reference forms edge conductivities only for node indices 2..size (F:258-269)
        mask = np.zeros(se.shape, bool)
        mask[1:xs if a != 0 else xs, 1:ys if a != 1 else ys, 1:zs if a != 2 else zs] = True
        if a == 0:
            mask[0] = False
        elif a == 1:
            mask[:, 0] = False
        else:
            mask[:, :, 0] = False
        out.append(np.where(mask, se, 0.0))
    return out


def _v_block(inp, x):
    Nx, Ny, Nz = inp.xs + 1, inp.ys + 1, inp.zs + 1
    oV = len(x) - Nx * Ny * Nz
    return np.asarray(x[oV:]).reshape((Nx, Ny, Nz), order="F"), oV


def edge_current(inp, geom, x, esig=None):
    """sigma_edge * dV/dh on every edge: how V enters the A rows (F:595-607)."""
    V, _ = _v_block(inp, x)
    esig = esig if esig is not None else edge_sigma(inp, geom)
    d = (inp.dx, inp.dy, inp.dz)
    dv = [(V[1:] - V[:-1]) / d[0], (V[:, 1:] - V[:, :-1]) / d[1], (V[:, :, 1:] - V[:, :, :-1]) / d[2]]
    return np.concatenate([(esig[a] * dv[a]).ravel(order="F") for a in range(3)])


class GaugeFixer:
    """The conducting nodes of a geometry and its floating bodies (connected through conducting
    edges, touching no Dirichlet node); ``v_on_nodes(inp, x)`` returns V on the conducting nodes
    with each floating body's mean removed."""

    def __init__(self, inp, geom, esig=None):
        import scipy.sparse as sp
        from scipy.sparse.csgraph import connected_components
        Nx, Ny, Nz = inp.xs + 1, inp.ys + 1, inp.zs + 1
        Nn = Nx * Ny * Nz
        esig = esig if esig is not None else edge_sigma(inp, geom)
        idx = np.arange(Nn).reshape((Nx, Ny, Nz), order="F")
        src, dst = [], []
        pairs = ((idx[:-1], idx[1:]), (idx[:, :-1], idx[:, 1:]), (idx[:, :, :-1], idx[:, :, 1:]))
        for a in range(3):
            m = esig[a] > SIGMA_CONDUCTING
            src.append(pairs[a][0][m])
            dst.append(pairs[a][1][m])
        src, dst = np.concatenate(src), np.concatenate(dst)
        self.nodes = np.unique(np.concatenate([src, dst]))
        if self.nodes.size == 0:
            self.labels = np.zeros(0, np.int64)
            self.floating = np.zeros(0, bool)
            self.count = np.zeros(0)
            return
        # relabel the conducting nodes 0..m-1 and find the connected bodies
        loc = np.searchsorted(self.nodes, src), np.searchsorted(self.nodes, dst)
        m = self.nodes.size
        G = sp.coo_matrix((np.ones(src.size), loc), shape=(m, m)).tocsr()
        ncomp, self.labels = connected_components(G, directed=False)
        i, rest = self.nodes % Nx, self.nodes // Nx
        j, k = rest % Ny, rest // Ny
        dirichlet = (i <= 1) | (i >= Nx - 2) | (j <= 1) | (j >= Ny - 2) | (k <= 1) | (k >= Nz - 2)   # F:393-396
        grounded = np.zeros(ncomp, bool)
        grounded[self.labels[dirichlet]] = True
        self.floating = ~grounded
        self.count = np.bincount(self.labels, minlength=ncomp)

    def v_on_nodes(self, inp, x):
        V, _ = _v_block(inp, x)
        v = V.ravel(order="F")[self.nodes].astype(np.float64)
        if v.size == 0:
            return v
        mean = np.bincount(self.labels, weights=v) / self.count
        return v - np.where(self.floating[self.labels], mean[self.labels], 0.0)


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    nb = float(np.linalg.norm(b))
    d = float(np.linalg.norm(a - b))
    return d / nb if nb > 0 else d


def compare_states(inp, geom, x, xref, H=None, Href=None, fixer=None, esig=None):
    """rel-L2 of x against xref per block: A, gauge-fixed V, the edge current sigma grad V, the
    raw V, and H when both cube sets are given."""
    Nn = (inp.xs + 1) * (inp.ys + 1) * (inp.zs + 1)
    oV = len(x) - Nn
    esig = esig if esig is not None else edge_sigma(inp, geom)
    fixer = fixer if fixer is not None else GaugeFixer(inp, geom, esig)
    out = {"A": rel_l2(x[:oV], xref[:oV]),
           "V_gauge_fixed": rel_l2(fixer.v_on_nodes(inp, x), fixer.v_on_nodes(inp, xref)),
           "J": rel_l2(edge_current(inp, geom, x, esig), edge_current(inp, geom, xref, esig)),
           "V_raw": rel_l2(x[oV:], xref[oV:])}
    if H is not None and Href is not None:
        out["H"] = rel_l2(np.concatenate([np.ravel(h) for h in H]), np.concatenate([np.ravel(h) for h in Href]))
    return out
