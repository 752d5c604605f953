"""Flatten a channel network into finite-volume cells and faces, and derive the
cell and face cross-sections (host-side setup of the 1-D network kernel).

Follows the reference's cell numbering so that states can be compared index by
index (hydrointel/solver/swe1d.py:113-166 ``build_topology``; sections
:204-215): junction cells first, then each reach's nodes followed by the ghost
cells of its non-junction ends; faces are the reach-internal faces, then the
upstream-end face, then the downstream-end face, reach by reach.

Cell kinds: 0 reach node, 1 junction (level pool), 2 inflow ghost, 3 stage
ghost, 4 closed ghost.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .channels import ChannelNetwork

KIND_REACH, KIND_JUNCTION, KIND_INFLOW, KIND_STAGE, KIND_CLOSED = 0, 1, 2, 3, 4
_END_KIND = {"inflow": KIND_INFLOW, "stage": KIND_STAGE, "closed": KIND_CLOSED}


@dataclass
class Topology:
    n_cells: int
    kind: np.ndarray
    reach_of: np.ndarray
    ghost_src: np.ndarray
    ghost_sign: np.ndarray
    face_l: np.ndarray
    face_r: np.ndarray
    z: np.ndarray
    b: np.ndarray
    m: np.ndarray
    zbank: np.ndarray
    n: np.ndarray
    dx: np.ndarray
    x: np.ndarray
    y: np.ndarray
    chain: np.ndarray

    @property
    def n_faces(self) -> int:
        return len(self.face_l)


def build_topology(net: ChannelNetwork) -> Topology:
    rows: list[tuple] = []     # (kind, reach, gsrc, gsign, z, b, m, zbank, n, dx, x, y, chain)
    fl: list[int] = []
    fr: list[int] = []

    def cell(*vals) -> int:
        rows.append(vals)
        return len(rows) - 1

    jcells = [cell(KIND_JUNCTION, -1, -1, 0, j.bed, j.width, j.side_slope, j.z_bank, j.manning, j.length, j.x, j.y,
                   0.0) for j in net.junctions]
    for ri, r in enumerate(net.reaches):
        ds, ch = r.spacing, r.chainage
        ids = [cell(KIND_REACH, ri, -1, 0, r.bed[k], r.width[k], r.side_slope[k], r.z_bank[k], r.manning[k], ds[k],
                    r.x[k], r.y[k], ch[k]) for k in range(r.n)]
        for a, b in zip(ids[:-1], ids[1:]):
            fl.append(a)
            fr.append(b)
        for end, inner, sign in ((r.up, ids[0], -1), (r.down, ids[-1], +1)):
            if end[0] == "junction":
                other = jcells[end[1]]
            else:
                k = 0 if sign < 0 else r.n - 1
                other = cell(_END_KIND[end[0]], ri, inner, sign, r.bed[k], r.width[k], r.side_slope[k], r.z_bank[k],
                             r.manning[k], ds[k], r.x[k], r.y[k], ch[k])
            if sign < 0:
                fl.append(other)
                fr.append(inner)
            else:
                fl.append(inner)
                fr.append(other)
    cols = list(zip(*rows))
    ints = [np.asarray(c, dtype=np.int64) for c in cols[:4]]
    flts = [np.asarray(c, dtype=np.float64) for c in cols[4:]]
    return Topology(len(rows), ints[0], ints[1], ints[2], ints[3], np.asarray(fl, dtype=np.int64),
                    np.asarray(fr, dtype=np.int64), *flts)


def sections(topo: Topology, slot_width_frac: float, z: np.ndarray | None = None, b: np.ndarray | None = None):
    """Cell sections (b, m, yb, ts) and face sections (fb, fm, fyb, fts).

    Bankfull depth yb = max(zbank - z, 0.2); above the bank the section continues
    as vertical walls of width ts = slot_width_frac * bankfull top width.  A face
    takes the mean bottom width and side slope of its two cells and bankfull depth
    max(mean bank - max(z_L, z_R), 0.1).  ``z``/``b`` may carry a member axis."""
    z = np.asarray(topo.z if z is None else z, dtype=np.float64)
    b = np.asarray(topo.b if b is None else b, dtype=np.float64)
    m, zbank = topo.m, topo.zbank
    yb = np.maximum(zbank - z, 0.2)
    ts = slot_width_frac * (b + 2 * m * yb)
    fl, fr = topo.face_l, topo.face_r
    zf = np.maximum(z[..., fl], z[..., fr])
    bank_f = 0.5 * (zbank[fl] + zbank[fr])
    ybf = np.maximum(bank_f - zf, 0.1)
    bf, mf = 0.5 * (b[..., fl] + b[..., fr]), 0.5 * (m[fl] + m[fr])
    tsf = slot_width_frac * (bf + 2 * mf * ybf)
    full = lambda a, ref: np.ascontiguousarray(np.broadcast_to(a, ref.shape), dtype=np.float64)
    return {"b": full(b, z), "m": full(m, z), "yb": full(yb, z), "ts": full(ts, z),
            "fb": full(bf, zf), "fm": full(mf, zf), "fyb": full(ybf, zf), "fts": full(tsf, zf)}


def bank_area(sec: dict) -> np.ndarray:
    return sec["yb"] * (sec["b"] + sec["m"] * sec["yb"])
