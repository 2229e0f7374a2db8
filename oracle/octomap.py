"""Octomap map files for the oracle: a pure-Python restatement of the reader amcl3d
uses (openOcTree + computePointCloud, amcl3d/src/PointCloudTools.cpp:26-82) and a
writer for test maps.  TEST INFRASTRUCTURE ONLY (the checker of the library's
native reader, never a fallback for it).

octomap is a third-party dependency whose source is not in the reference tree
(package.xml lists octomap_ros without a version; the README targets ROS Kinetic,
whose octomap is 1.8.x).  Restated from its published file formats:

* header: a first line starting "# Octomap OcTree binary file" (.bt) or
  "# Octomap OcTree file" (.ot), then whitespace-separated tokens: lines whose
  token starts with '#' are comments, "id <type>", "size <nodes>", "res <m>",
  unknown keywords skip their line, "data" ends the header (rest of its line
  skipped); id "1" is the deprecated name of "OcTree"; id must be set, res > 0.
* .bt body (OcTree::readBinaryNode): per inner node two bytes, children 0-3 then
  4-7, two bits per child i at bit positions 2i (lo) and 2i+1 (hi):
  lo=1,hi=0 free leaf; lo=0,hi=1 occupied leaf; lo=1,hi=1 inner node (its own
  two bytes follow, depth first, in child order); 0,0 no child.  The tree must
  have as many nodes as the header's size.
* .ot body (readNodesRecurs): per node its float32 log-odds, one byte whose bit i
  says child i exists, then the existing children, depth first.  A node without
  children is a leaf, occupied when its log-odds is >= 0 (probability 0.5).
* geometry: 16 levels, root key 32768 per axis; child i at depth d has the key
  parent + off if bit (i>>axis)&1 else parent - off - (off == 0), off = 32768 >> d;
  a leaf centre is (key - 32768 + 0.5) * res at depth 16, else
  (floor((key - 32768) / 2^(16-d)) + 0.5) * res * 2^(16-d); leaves are visited
  depth first in child order (the leaf iterator's order).
* computePointCloud: the float centres of the occupied leaves; metric min/max over
  every leaf (free ones too): min of centre - size/2, max of (centre - size/2) + size.
"""

from __future__ import annotations

import math
import struct
from pathlib import Path

import numpy as np

DEPTH = 16
ROOT_KEY = 32768
BT_HEADER = "# Octomap OcTree binary file"
OT_HEADER = "# Octomap OcTree file"


class OctomapError(RuntimeError):
    pass


def key_to_coord(key: int, depth: int, res: float) -> float:
    if depth == 0:
        return 0.0
    if depth == DEPTH:
        return (float(key - ROOT_KEY) + 0.5) * res
    span = float(1 << (DEPTH - depth))
    return (math.floor((float(key) - float(ROOT_KEY)) / span) + 0.5) * (res * span)


def _child_key(key, i, depth):
    off = ROOT_KEY >> depth
    return tuple(key[a] + off if (i >> a) & 1 else key[a] - off - (0 if off else 1) for a in range(3))


def _parse_header(b: bytes, first: str):
    nl = b.find(b"\n")
    if nl < 0 or not b[:nl].decode("latin-1").startswith(first):
        raise OctomapError("first line is not an octomap header")
    pos = nl + 1
    ident, size, res = "", 0, 0.0

    def token(p):
        while p < len(b) and chr(b[p]).isspace():
            p += 1
        q = p
        while q < len(b) and not chr(b[q]).isspace():
            q += 1
        return b[p:q].decode("latin-1"), q

    def skip_line(p):
        q = b.find(b"\n", p)
        return len(b) if q < 0 else q + 1

    while True:
        tok, pos = token(pos)
        if tok == "":
            raise OctomapError("header without data")
        if tok == "data":
            pos = skip_line(pos)
            break
        if tok.startswith("#"):
            pos = skip_line(pos)
        elif tok == "id":
            ident, pos = token(pos)
        elif tok == "res":
            v, pos = token(pos)
            res = float(v)
        elif tok == "size":
            v, pos = token(pos)
            size = int(v)
        else:
            pos = skip_line(pos)
    if ident == "1":
        ident = "OcTree"
    if ident == "" or not res > 0.0:
        raise OctomapError("header without id or with res <= 0")
    return ident, size, res, pos


class _Acc:
    def __init__(self, res):
        self.res = res
        self.occ = []
        self.mn = [math.inf] * 3
        self.mx = [-math.inf] * 3
        self.nodes = 1  # the root

    def leaf(self, key, depth, occupied):
        c = [key_to_coord(key[a], depth, self.res) for a in range(3)]
        size = self.res * float(1 << (DEPTH - depth))
        half = size / 2.0
        for a in range(3):
            lo = c[a] - half
            self.mn[a] = min(self.mn[a], lo)
            self.mx[a] = max(self.mx[a], lo + size)
        if occupied:
            self.occ.append(c)


def _read_bt(b, pos, acc):
    stack = [((ROOT_KEY,) * 3, 0, None)]
    # explicit depth-first recursion in child order
    def node(key, depth):
        nonlocal pos
        if depth >= DEPTH:
            raise OctomapError("inner node below the last level")
        if pos + 2 > len(b):
            raise OctomapError("truncated tree")
        lo4, hi4 = b[pos], b[pos + 1]
        pos += 2
        kinds = []
        for i in range(8):
            byte = lo4 if i < 4 else hi4
            j = i % 4
            kinds.append(((byte >> (2 * j)) & 1, (byte >> (2 * j + 1)) & 1))
        for i, (l, h) in enumerate(kinds):
            if (l, h) == (0, 0):
                continue
            acc.nodes += 1
            ck = _child_key(key, i, depth + 1)
            if (l, h) == (1, 0):
                acc.leaf(ck, depth + 1, False)
            elif (l, h) == (0, 1):
                acc.leaf(ck, depth + 1, True)
            else:
                node(ck, depth + 1)

    del stack
    node((ROOT_KEY,) * 3, 0)
    return pos


def _read_ot(b, pos, acc):
    def node(key, depth):
        nonlocal pos
        if pos + 5 > len(b):
            raise OctomapError("truncated tree")
        (lo,) = struct.unpack_from("<f", b, pos)
        ch = b[pos + 4]
        pos += 5
        if ch == 0:
            if depth == 0:
                acc.leaf(key, 0, lo >= 0.0)
            return lo
        if depth >= DEPTH:
            raise OctomapError("inner node below the last level")
        for i in range(8):
            if (ch >> i) & 1:
                acc.nodes += 1
                ck = _child_key(key, i, depth + 1)
                v = node(ck, depth + 1)
                if v is not None:
                    acc.leaf(ck, depth + 1, v >= 0.0)
        return None

    node((ROOT_KEY,) * 3, 0)
    return pos


def read(path) -> dict:
    """openOcTree + computePointCloud: {points (n, 3) float32, min, max, res, nodes}.
    Raises OctomapError where the reference throws std::runtime_error."""
    path = str(path)
    if len(path) < 3:
        raise OctomapError("path shorter than its extension")
    if not Path(path).exists():
        raise OctomapError("Cannot find file " + path)
    b = Path(path).read_bytes()
    if path.endswith(".bt"):
        ident, size, res, pos = _parse_header(b, BT_HEADER)
        if ident != "OcTree":
            raise OctomapError("not an OcTree")
        acc = _Acc(res)
        if size > 0:
            _read_bt(b, pos, acc)
        else:
            acc.nodes = 0
        if acc.nodes != size:
            raise OctomapError("tree size differs from the header")
    elif path.endswith(".ot"):
        ident, size, res, pos = _parse_header(b, OT_HEADER)
        if ident != "OcTree":
            raise OctomapError("not an OcTree")
        acc = _Acc(res)
        if size > 0:
            _read_ot(b, pos, acc)
        else:
            acc.nodes = 0
    else:
        raise OctomapError("OcTree cannot be created from file " + path)
    if acc.nodes <= 1:
        raise OctomapError("OcTree is empty")
    pts = np.array(acc.occ, dtype=np.float64).reshape(-1, 3).astype(np.float32)
    return {"points": pts, "min": tuple(acc.mn), "max": tuple(acc.mx), "res": res, "nodes": acc.nodes}


# ---- writer of test maps -------------------------------------------------------------------------

def coord_to_key(c: float, res: float) -> int:
    """octomap's coordToKey at full depth: floor(c / res) + 32768."""
    return int(math.floor(c / res)) + ROOT_KEY


def _build(leaves):
    """Nested dict tree from {(key, depth): occupied}: a node is a dict child -> node,
    a leaf is a bool."""
    root = {}
    for (key, depth), occ in leaves.items():
        node = root
        for d in range(1, depth + 1):
            off = ROOT_KEY >> d
            i = 0
            for a in range(3):
                # the child whose key range holds `key`
                shift = DEPTH - d
                bit = ((key[a]) >> shift) & 1
                i |= bit << a
            del off
            if d == depth:
                node[i] = bool(occ)
            else:
                node = node.setdefault(i, {})
                if not isinstance(node, dict):
                    raise ValueError("a leaf above another leaf")
    return root


def _count(node):
    return 1 + sum(_count(c) if isinstance(c, dict) else 1 for c in node.values())


def write_bt(path, leaves: dict, res: float, extra_header: str = "") -> int:
    """leaves: {((kx, ky, kz), depth): occupied}; keys are full-depth keys of any
    point inside the leaf.  Returns the node count written in the header."""
    root = _build(leaves)
    out = bytearray()

    def emit(node):
        b = [0, 0]
        for i in range(8):
            if i not in node:
                continue
            c = node[i]
            lo, hi = (1, 1) if isinstance(c, dict) else ((0, 1) if c else (1, 0))
            b[i // 4] |= (lo << (2 * (i % 4))) | (hi << (2 * (i % 4) + 1))
        out.extend(bytes(b))
        for i in range(8):
            if isinstance(node.get(i), dict):
                emit(node[i])

    emit(root)
    n = _count(root)
    head = f"{BT_HEADER}\n# written by the test map writer\n{extra_header}id OcTree\nsize {n}\nres {res!r}\ndata\n"
    Path(path).write_bytes(head.encode() + bytes(out))
    return n


def write_ot(path, leaves: dict, res: float, occ_lo=0.85, free_lo=-0.4) -> int:
    """Same tree in the .ot layout (log-odds per node; inner nodes carry the maximum
    of their children, as octomap's updateInnerOccupancy leaves them)."""
    root = _build(leaves)
    out = bytearray()

    def value(node):
        if isinstance(node, dict):
            return max(value(c) for c in node.values())
        return occ_lo if node else free_lo

    def emit(node):
        out.extend(struct.pack("<f", value(node)))
        mask = 0
        if isinstance(node, dict):
            for i in node:
                mask |= 1 << i
        out.append(mask)
        if isinstance(node, dict):
            for i in range(8):
                if i in node:
                    emit(node[i])

    emit(root)
    n = _count(root)
    Path(path).write_bytes(f"{OT_HEADER}\nid OcTree\nsize {n}\nres {res!r}\ndata\n".encode() + bytes(out))
    return n


def leaves_from_points(points, res: float, occupied=True) -> dict:
    """Full-depth leaves holding the given coordinates."""
    out = {}
    for p in np.asarray(points, dtype=np.float64):
        out[(tuple(coord_to_key(float(v), res) for v in p[:3]), DEPTH)] = occupied
    return out
