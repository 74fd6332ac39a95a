"""Restatement of the reference's `.tree` output with the adaptive indexer (test infrastructure
only): ExteriorPoissonRecon's Execute (ExteriorPoissonRecon/ExteriorPoissonRecon.cpp:259-270) with
HierarchicalAdaptedIndexer::write (Include/Hat.adaptive.inl:399-405).

    file    = u32 dim | u64 typeid(HierarchicalAdaptedIndexer<dim>).hash_code() | XForm<double, dim+1>
              raw (one 8-byte word that is not matrix data, then (dim+1)^2 doubles) | x | y | tree |
              activeSizes | functionNodes | elementNodes
    x, y    = u64 levels, then per level i64 n and n doubles (the level's coefficients in the
              indexer's function order)
    tree    = the root, then, depth first, for every node that has children its 2^dim children in one
              block before the subtrees of those children (child c has offset 2 O + bit d of c on
              axis d; Misha/RegularTree.inl:615-642)
    node    = RegularTreeNode<dim, NodeData, unsigned short> raw: u16 depth, u16 offset[dim], padding
              to 8 (3D) / 16 (4D) bytes, parent pointer, children pointer (only tested against null
              when read back), u64 functionIndex, u64 elementIndex (-1 when none): 40 / 48 bytes
    activeSizes = u64 count, then count u64 (active functions per level)
    functionNodes, elementNodes = u64 levels, then per level u64 n and n pointers (the reader
              replaces them, Hat.adaptive.inl:376-397, so only the counts carry information)

A tree node of depth t >= 1 and offset O is the function of level t-1 with offset O when
0 <= O <= 2^(t-1) and the element of level t-1 with offset O when 0 <= O < 2^(t-1).  The tree holds
the nodes the indexer created: the root and its children, and the children of every node that is
the parent of a node in (a) the (K, K+1) window of a sample cell's ancestor at some depth
(Hat.adaptive.inl:583-604) or (b) the one-ring window of an ancestor of an active function at some
depth (Hat.adaptive.inl:676-701).
"""
from __future__ import annotations

import struct

import numpy as np

HASH = {3: 0xf40c6f40c49db503, 4: 0xfb48bf69bf639a05}


def layout(dim: int):
    """(node bytes, byte offset of the parent pointer, byte offset of the node data)."""
    ptr = 8 if dim == 3 else 16
    return ptr + 32, ptr, ptr + 16


def parse(raw: bytes) -> dict:
    """Every part of an adaptive `.tree`: dim, hash, xform, x / y per level, the nodes in file order
    (depth, offset, has_children, findex, eindex; the byte offset of each record in `rec_at`),
    active / function / element counts per level and the byte ranges of the pointer words."""
    o = 0
    dim, hsh = struct.unpack_from("<IQ", raw, o)
    o += 12
    xf = np.frombuffer(raw, "<f8", (dim + 1) ** 2, o + 8).copy()
    o += 8 + 8 * (dim + 1) ** 2
    coef = []
    for _ in range(2):
        (L,) = struct.unpack_from("<Q", raw, o)
        o += 8
        lv = []
        for _ in range(L):
            (n,) = struct.unpack_from("<q", raw, o)
            lv.append(np.frombuffer(raw, "<f8", n, o + 8).copy())
            o += 8 + 8 * n
        coef.append(lv)
    node, ptr, dat = layout(dim)
    recs = []

    def read_node():
        nonlocal o
        recs.append(o)
        o += node
        return recs[-1]

    root = read_node()
    stack = [root]
    while stack:
        at = stack.pop()
        if struct.unpack_from("<Q", raw, at + ptr + 8)[0] == 0:
            continue
        block = [read_node() for _ in range(1 << dim)]
        stack.extend(reversed(block))
    # the file lists a block's children right after their parent's block is read depth first, which
    # is what the stack above replays (children pushed in reverse so child 0's subtree comes first)
    rec = np.frombuffer(raw, np.uint8).reshape(-1)
    at = np.array(recs)
    R = np.stack([rec[a:a + node] for a in at])
    depth = R[:, 0:2].copy().view("<u2")[:, 0].astype(np.int64)
    offset = R[:, 2:2 + 2 * dim].copy().view("<u2").astype(np.int64)
    has = R[:, ptr + 8:ptr + 16].copy().view("<u8")[:, 0] != 0
    fe = R[:, dat:dat + 16].copy().view("<i8")
    (na,) = struct.unpack_from("<Q", raw, o)
    active = np.frombuffer(raw, "<u8", na, o + 8).astype(np.int64)
    o += 8 + 8 * na
    counts, ptr_ranges = [], []
    for _ in range(2):
        (L,) = struct.unpack_from("<Q", raw, o)
        o += 8
        c = []
        for _ in range(L):
            (n,) = struct.unpack_from("<Q", raw, o)
            c.append(n)
            ptr_ranges.append((o + 8, o + 8 + 8 * n))
            o += 8 + 8 * n
        counts.append(np.array(c))
    if o != len(raw):
        raise ValueError(f"{len(raw) - o} trailing bytes")
    return {"dim": dim, "hash": hsh, "xform": xf, "x": coef[0], "y": coef[1], "rec_at": at, "depth": depth,
            "offset": offset, "has_children": has, "findex": fe[:, 0], "eindex": fe[:, 1], "active": active,
            "functions": counts[0], "elements": counts[1], "ptr_ranges": ptr_ranges}


def masked(raw: bytes) -> np.ndarray:
    """The file's bytes with the words that hold memory addresses there (node parent and children
    pointers, function / element node pointers) and node padding zeroed, the children word reduced
    to 0 / 1 and the XForm's leading word zeroed: two files that agree here agree in every byte the
    reference's reader interprets."""
    t = parse(raw)
    b = np.frombuffer(raw, np.uint8).copy()
    dim = t["dim"]
    node, ptr, _ = layout(dim)
    b[12:20] = 0
    for a, has in zip(t["rec_at"], t["has_children"]):
        b[a + 2 + 2 * dim:a + ptr + 16] = 0
        b[a + ptr + 8] = 1 if has else 0
    for lo, hi in t["ptr_ranges"]:
        b[lo:hi] = 0
    return b


def refinement(dim: int, depth: int, K: int, cells: np.ndarray, fnodes, nactive) -> list:
    """has-children flags per tree depth t = 0 .. depth+1 ((2^t)^dim bytes, axis 0 most
    significant) of the indexer's tree, from the sample cells (finest level, (m, dim)) and the
    active functions of every level (fnodes[l][:nactive[l]], nodes of the (2^l+1)^dim grid)."""
    marks = [np.zeros((1 << t,) * dim, bool) for t in range(depth + 2)]
    cells = np.asarray(cells, np.int64).reshape(-1, dim)

    def mark(t, lo, hi):
        side = 1 << t
        lo = np.clip(lo, 0, side - 1)
        hi = np.clip(hi, 0, side - 1)
        for a, b in zip(lo, hi):
            if (a > b).any():
                continue
            marks[t][tuple(slice(int(a[k]), int(b[k]) + 1) for k in range(dim))] = True

    for t in range(1, depth + 2):
        A = cells >> (depth + 1 - t)
        mark(t, A - K, A + K + 1)
    for l in range(depth + 1):
        r1 = (1 << l) + 1
        I = np.stack(np.unravel_index(np.asarray(fnodes[l][:nactive[l]], np.int64), (r1,) * dim), axis=1)
        for t in range(1, l + 2):
            B = I >> (l + 1 - t)
            mark(t, B - 1, B + 1)
    refined = [np.ones(1, np.uint8)]
    for t in range(1, depth + 2):
        side = 1 << t
        flags = np.zeros((side,) * dim, np.uint8)
        if t <= depth:
            m = marks[t + 1]
            # a node has children when one of its children is marked
            flags = m.reshape(tuple(x for _ in range(dim) for x in (side, 2))).any(axis=tuple(range(1, 2 * dim, 2)))
        refined.append(flags.astype(np.uint8).ravel())
    return refined


def node_indices(dim: int, depth: np.ndarray, offset: np.ndarray, fnodes, enodes):
    """functionIndex and elementIndex of every tree node (-1 when none) from the level tables."""
    fi = np.full(len(depth), -1, np.int64)
    ei = np.full(len(depth), -1, np.int64)
    for l in range(len(fnodes)):
        r = 1 << l
        sel = depth == l + 1
        O = offset[sel]
        fmap = np.full((r + 1) ** dim, -1, np.int64)
        fmap[np.asarray(fnodes[l], np.int64)] = np.arange(len(fnodes[l]))
        emap = np.full(r ** dim, -1, np.int64)
        emap[np.asarray(enodes[l], np.int64)] = np.arange(len(enodes[l]))
        f = np.full(len(O), -1, np.int64)
        e = np.full(len(O), -1, np.int64)
        inF = (O <= r).all(axis=1)
        inE = (O < r).all(axis=1)
        f[inF] = fmap[np.ravel_multi_index(O[inF].T, (r + 1,) * dim)]
        e[inE] = emap[np.ravel_multi_index(O[inE].T, (r,) * dim)]
        fi[sel] = f
        ei[sel] = e
    return fi, ei
