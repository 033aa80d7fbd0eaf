"""Reader, walker and structural differ for the .octree / .octreenodes / .octreedata files.

Layouts (octree_io.h:48-83, Node.h:16-18, VoxelData.h:9-13):

* node record, 24 bytes: ``u64 data``, ``u64 children_base``, ``i8 children_offset[8]``
  (-1 = no child); a child's index is ``children_base + children_offset[k]``;
* data record, 32 bytes: ``u64 morton``, ``f32 color[3]``, ``f32 normal[3]``;
* header text: ``#octreeheader 1`` / ``gridlength`` / ``n_nodes`` / ``n_data`` / ``END``.

The root is the last node record.  Floating-point fields are compared as bit patterns
except that any two NaNs compare equal: the bits of a NaN produced by 0 * inf or by NaN
propagation differ between x86-64, AArch64 and the GPU, including between builds of the
reference itself.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

NODE_DTYPE = np.dtype([("data", "<u8"), ("children_base", "<u8"), ("children_offset", "i1", (8,))])
DATA_DTYPE = np.dtype([("morton", "<u8"), ("color", "<f4", (3,)), ("normal", "<f4", (3,))])
assert NODE_DTYPE.itemsize == 24 and DATA_DTYPE.itemsize == 32


@dataclass
class Octree:
    gridlength: int
    nodes: np.ndarray  # NODE_DTYPE
    data: np.ndarray   # DATA_DTYPE


def parse_header(path: str) -> dict:
    """parseOctreeHeader (octree_io.h:86-110)."""
    with open(path) as f:
        toks = f.read().split()
    if len(toks) < 2 or toks[0] != "#octreeheader":
        raise ValueError("not an octree header: %s" % path)
    out = {"version": int(toks[1])}
    i = 2
    while i < len(toks):
        t = toks[i]
        if t == "END":
            break
        if t in ("gridlength", "n_nodes", "n_data"):
            out[t] = int(toks[i + 1])
            i += 2
        else:
            i += 1
    return out


def header_text(gridlength: int, n_nodes: int, n_data: int) -> str:
    """writeOctreeHeader (octree_io.h:74-83)."""
    return "#octreeheader 1\ngridlength %d\nn_nodes %d\nn_data %d\nEND\n" % (gridlength, n_nodes, n_data)


def read_octree(base: str) -> Octree:
    """Read ``<base>.octree`` (+ nodes, data)."""
    h = parse_header(base + ".octree")
    nodes = np.fromfile(base + ".octreenodes", dtype=NODE_DTYPE)
    data = np.fromfile(base + ".octreedata", dtype=DATA_DTYPE)
    if nodes.shape[0] != h["n_nodes"] or data.shape[0] != h["n_data"]:
        raise ValueError("octree files disagree with the header")
    return Octree(h["gridlength"], nodes, data)


def from_bytes(gridlength: int, node_bytes: bytes, data_bytes: bytes) -> Octree:
    return Octree(gridlength, np.frombuffer(node_bytes, dtype=NODE_DTYPE),
                  np.frombuffer(data_bytes, dtype=DATA_DTYPE))


def write_octree(base: str, tree: Octree) -> None:
    d = os.path.dirname(base)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(base + ".octree", "w") as f:
        f.write(header_text(tree.gridlength, tree.nodes.shape[0], tree.data.shape[0]))
    tree.nodes.tofile(base + ".octreenodes")
    tree.data.tofile(base + ".octreedata")


def leaves(tree: Octree):
    """Walk from the root and return (morton codes, data indices) of all leaves, in Morton order."""
    n = tree.nodes
    if n.shape[0] == 0:
        return np.zeros(0, np.uint64), np.zeros(0, np.uint64)
    depth = int(tree.gridlength).bit_length() - 1
    out_m, out_d = [], []
    stack = [(n.shape[0] - 1, 0, 0)]
    while stack:
        idx, level, prefix = stack.pop()
        rec = n[idx]
        offs = rec["children_offset"]
        if level == depth:
            if rec["data"] != 0 or (offs != -1).any():
                out_m.append(prefix)
                out_d.append(int(rec["data"]))
            continue
        for k in range(7, -1, -1):
            if offs[k] != -1:
                stack.append((int(rec["children_base"]) + int(offs[k]), level + 1, (prefix << 3) | k))
    return np.array(out_m, np.uint64), np.array(out_d, np.uint64)


def _float_fields_equal(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Row-wise equality of float32 arrays by bit pattern, any NaN equal to any NaN."""
    ai = a.view(np.uint32)
    bi = b.view(np.uint32)
    same = ai == bi
    both_nan = np.isnan(a) & np.isnan(b)
    return (same | both_nan).reshape(a.shape[0], -1).all(axis=1)


def diff(a: Octree, b: Octree, max_report: int = 5) -> list:
    """Structural comparison; returns a list of human-readable differences (empty if equal)."""
    out = []
    if a.gridlength != b.gridlength:
        out.append("gridlength %d != %d" % (a.gridlength, b.gridlength))
    if a.nodes.shape[0] != b.nodes.shape[0]:
        out.append("n_nodes %d != %d" % (a.nodes.shape[0], b.nodes.shape[0]))
    if a.data.shape[0] != b.data.shape[0]:
        out.append("n_data %d != %d" % (a.data.shape[0], b.data.shape[0]))
    n = min(a.nodes.shape[0], b.nodes.shape[0])
    if n:
        av = a.nodes[:n].view(np.uint8).reshape(n, 24)
        bv = b.nodes[:n].view(np.uint8).reshape(n, 24)
        bad = np.nonzero((av != bv).any(axis=1))[0]
        for i in bad[:max_report]:
            out.append("node %d: %s != %s" % (i, a.nodes[i], b.nodes[i]))
        if bad.size > max_report:
            out.append("... %d differing nodes" % bad.size)
    m = min(a.data.shape[0], b.data.shape[0])
    if m:
        mort = a.data["morton"][:m] == b.data["morton"][:m]
        col = _float_fields_equal(a.data["color"][:m], b.data["color"][:m])
        nor = _float_fields_equal(a.data["normal"][:m], b.data["normal"][:m])
        bad = np.nonzero(~(mort & col & nor))[0]
        for i in bad[:max_report]:
            out.append("data %d: %s != %s" % (i, a.data[i], b.data[i]))
        if bad.size > max_report:
            out.append("... %d differing data records" % bad.size)
    return out


def equal(a: Octree, b: Octree) -> bool:
    return not diff(a, b, max_report=1)


CANONICAL_NAN = np.uint32(0x7FC00000)


def digest(tree: Octree) -> dict:
    """SHA-256 of the node and data files, with every NaN in the data records' colour and
    normal replaced by one quiet-NaN pattern first, so two trees have the same digest
    exactly when `diff` finds them equal (up to hash collisions)."""
    import hashlib

    data = tree.data.copy()
    for field in ("color", "normal"):
        f = data[field]
        bits = f.view(np.uint32)
        bits[np.isnan(f)] = CANONICAL_NAN
    return {"gridlength": int(tree.gridlength), "n_nodes": int(tree.nodes.shape[0]),
            "n_data": int(tree.data.shape[0]),
            "nodes_sha256": hashlib.sha256(np.ascontiguousarray(tree.nodes).tobytes()).hexdigest(),
            "data_sha256": hashlib.sha256(data.tobytes()).hexdigest()}


class StreamDigest:
    """`digest` of an octree whose node and data files arrive in pieces, in file order
    (a build's sink, or files read in chunks), without holding them: the same hashes
    as ``digest(tree)`` of the whole files."""

    def __init__(self, gridlength: int):
        import hashlib
        self.gridlength = int(gridlength)
        self._h = {0: hashlib.sha256(), 1: hashlib.sha256()}
        self._n = {0: 0, 1: 0}
        self._tail = b""  # bytes of a data record split between two pieces
        self.nan_fields = 0

    def update(self, kind: int, piece) -> None:
        """Append `piece` (bytes-like) to the node file (kind 0) or the data file (kind 1)."""
        if kind == 0:
            self._h[0].update(piece)
            self._n[0] += len(piece)
            return
        b = self._tail + bytes(piece)
        whole = len(b) // DATA_DTYPE.itemsize * DATA_DTYPE.itemsize
        self._tail = b[whole:]
        if whole:
            data = np.frombuffer(b[:whole], dtype=DATA_DTYPE).copy()
            for field in ("color", "normal"):
                f = data[field]
                m = np.isnan(f)
                self.nan_fields += int(m.sum())
                f.view(np.uint32)[m] = CANONICAL_NAN
            self._h[1].update(data.tobytes())
            self._n[1] += whole

    def result(self) -> dict:
        if self._tail or self._n[0] % NODE_DTYPE.itemsize:
            raise ValueError("octree files end inside a record")
        return {"gridlength": self.gridlength, "n_nodes": self._n[0] // NODE_DTYPE.itemsize,
                "n_data": self._n[1] // DATA_DTYPE.itemsize, "nodes_sha256": self._h[0].hexdigest(),
                "data_sha256": self._h[1].hexdigest()}


def file_digest(base: str, chunk: int = 64 << 20) -> dict:
    """`digest` of the octree files at `base`, read in chunks (for files too large to load)."""
    h = parse_header(base + ".octree")
    d = StreamDigest(h["gridlength"])
    for kind, ext in ((0, ".octreenodes"), (1, ".octreedata")):
        with open(base + ext, "rb") as f:
            while True:
                b = f.read(chunk)
                if not b:
                    break
                d.update(kind, b)
    out = d.result()
    if out["n_nodes"] != h["n_nodes"] or out["n_data"] != h["n_data"]:
        raise ValueError("octree files disagree with the header")
    return out
