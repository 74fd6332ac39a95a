"""Restatement of the reference's `.density.tree` output (test infrastructure only): what
ExteriorPoissonRecon writes after the solve (ExteriorPoissonRecon/ExteriorPoissonRecon.cpp:272-277)
with TreeEstimator::write (Include/GridSamples.inl:734-738) and RegularTreeNode::write in its
non-serialised form (Misha/RegularTree.inl:615-642).

    file    = XForm<double, dim+1> written raw (one 8-byte word that is not matrix data, then the
              (dim+1)^2 doubles) | nodes | targetSamplesPerCell (double, 2^(dim-2))
    nodes   = the root, then, depth first, for every node that has children its 2^dim children in
              one block, before the subtrees of those children (child c has offset 2 O + bit d of c
              on axis d)
    node    = RegularTreeNode<dim, DensityAndNoiseInfo<dim>, unsigned short> written raw:
              u16 depth, u16 offset[dim], padding to 8 bytes (3D) / 16 bytes (4D), parent pointer,
              children pointer (only whether it is null is read back, RegularTree.inl:649-660),
              weightSum, positionSum[dim], 8 bytes of padding, covarianceSum[dim][dim]
              (GridSamples.h:79-94): 136 bytes in 3D, 208 in 4D

A node of tree depth t >= 1 whose offset lies inside [0, 2^(t-1)]^dim holds the splatted density of
the regular vertex with those coordinates at resolution 2^(t-1) (the estimator's level t-1);
the root and the nodes outside hold zeros.  Which nodes have children is the density tree's
refinement (one flag per depth-t cell, axis 0 most significant).
"""
from __future__ import annotations

import struct

import numpy as np


def layout(dim: int):
    """(node bytes, byte offset of the parent pointer, byte offset of the data) of one node."""
    ptr = 8 if dim == 3 else 16
    data = ptr + 16
    return data + 8 * (1 + dim + 1 + dim * dim), ptr, data


def parse(raw: bytes, dim: int) -> dict:
    """Nodes of a `.density.tree` as arrays: depth (n,), offset (n, dim), has_children (n,),
    data (n, 1 + dim + dim^2) (weight, position sum, covariance sum; the padding word dropped)."""
    node, ptr, dat = layout(dim)
    xf_bytes = 8 + 8 * (dim + 1) ** 2
    body = len(raw) - xf_bytes - 8
    if body < 0 or body % node:
        raise ValueError(f"size {len(raw)} is not an XForm, whole nodes and the trailer")
    n = body // node
    rec = np.frombuffer(raw, np.uint8, n * node, xf_bytes).reshape(n, node)
    depth = rec[:, 0:2].copy().view("<u2")[:, 0].astype(np.int64)
    offset = rec[:, 2:2 + 2 * dim].copy().view("<u2").astype(np.int64)
    children = rec[:, ptr + 8:ptr + 16].copy().view("<u8")[:, 0]
    words = rec[:, dat:].copy().view("<f8")
    data = np.concatenate([words[:, :1 + dim], words[:, 2 + dim:]], axis=1)
    return {"xform": np.frombuffer(raw, "<f8", (dim + 1) ** 2, 8).copy(), "depth": depth, "offset": offset,
            "has_children": children != 0, "data": data, "trailer": struct.unpack_from("<d", raw, len(raw) - 8)[0]}


def nodes(dim: int, refined) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Depth, offset and has-children flag of every node in file order, from the refinement flags
    refined[t] ((2^t)^dim bytes, t = 0 .. max depth; refined[0] is the root's)."""
    depth, offset, has = [0], [(0,) * dim], [bool(refined[0][0])]
    tmax = len(refined) - 1

    def flag(t, o):
        if t > tmax:
            return False
        side = 1 << t
        li = 0
        for d in range(dim):
            li = li * side + o[d]
        return bool(refined[t][li])

    stack = [(0, (0,) * dim)] if has[0] else []
    while stack:
        t, o = stack.pop()
        kids = [tuple(2 * o[d] + ((c >> d) & 1) for d in range(dim)) for c in range(1 << dim)]
        for k in kids:
            depth.append(t + 1)
            offset.append(k)
            has.append(flag(t + 1, k))
        for k in reversed(kids):
            if flag(t + 1, k):
                stack.append((t + 1, k))
    return np.array(depth), np.array(offset).reshape(-1, dim), np.array(has)


def node_data(dim: int, depth: np.ndarray, offset: np.ndarray, density) -> np.ndarray:
    """Each node's data from the estimator's regular levels density[l] ((2^l+1)^dim, 1+dim+dim^2)."""
    W = 1 + dim + dim * dim
    out = np.zeros((len(depth), W))
    for i, (t, o) in enumerate(zip(depth, offset)):
        if t == 0:
            continue
        r = 1 << (t - 1)
        if (o > r).any():
            continue
        idx = 0
        for d in range(dim):
            idx = idx * (r + 1) + int(o[d])
        out[i] = np.asarray(density[t - 1]).reshape(-1, W)[idx]
    return out


def serialize(dim: int, xform: np.ndarray, depth, offset, has_children, data) -> bytes:
    """A `.density.tree` with zero pointer and padding words and 1 as the children word of a node
    that has children."""
    node, ptr, dat = layout(dim)
    n = len(depth)
    rec = np.zeros((n, node), np.uint8)
    rec[:, 0:2] = np.asarray(depth, "<u2").reshape(n, 1).view(np.uint8)
    rec[:, 2:2 + 2 * dim] = np.ascontiguousarray(np.asarray(offset, "<u2")).view(np.uint8).reshape(n, 2 * dim)
    rec[:, ptr + 8:ptr + 16] = np.asarray(has_children, "<u8").reshape(n, 1).view(np.uint8)
    words = np.zeros((n, 2 + dim + dim * dim))
    words[:, :1 + dim] = data[:, :1 + dim]
    words[:, 2 + dim:] = data[:, 1 + dim:]
    rec[:, dat:] = words.astype("<f8").view(np.uint8)
    head = struct.pack("<Q", 0) + np.asarray(xform, "<f8").tobytes()
    return head + rec.tobytes() + struct.pack("<d", 2.0 ** (dim - 2))
