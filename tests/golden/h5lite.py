"""Minimal reader for the HDF5 files SpinParser writes (classic format: superblock v0,
v1 object headers, symbol-table groups with v1 B-trees and local heaps, contiguous or
compact datasets, attributes).  h5py is not available in this environment; this reader
covers exactly what the .obs / .ref / .checkpoint files contain (float32 datasets,
float32[3] array datasets, float32 attributes).

Test infrastructure: used to extract the reference's golden .ref data into fixtures and to
read the .obs files the package writes.
"""
from __future__ import annotations

import struct

import numpy as np


class H5Error(ValueError):
    pass


class _Reader:
    def __init__(self, data: bytes):
        self.b = data
        if data[:8] != b"\x89HDF\r\n\x1a\n":
            raise H5Error("not an HDF5 file")
        if data[8] != 0:
            raise H5Error(f"unsupported superblock version {data[8]}")
        self.so = data[13]
        self.sl = data[14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("only 8-byte offsets/lengths supported")
        # root group symbol table entry at 24 + 4*8 = 56
        self.root = self._symbol_entry(56)

    def u(self, off, n):
        return int.from_bytes(self.b[off:off + n], "little")

    def _symbol_entry(self, off):
        name_off = self.u(off, 8)
        header = self.u(off + 8, 8)
        cache = self.u(off + 16, 4)
        scratch = (self.u(off + 24, 8), self.u(off + 32, 8)) if cache == 1 else None
        return {"name_off": name_off, "header": header, "cache": cache, "scratch": scratch}

    def messages(self, addr):
        b = self.b
        if b[addr] != 1:
            raise H5Error(f"unsupported object header version {b[addr]} at {addr}")
        nmsg = self.u(addr + 2, 2)
        size = self.u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p < start + length and len(out) < nmsg:
                mtype = self.u(p, 2)
                msize = self.u(p + 2, 2)
                body = p + 8
                if mtype == 0x10:  # continuation
                    blocks.append((self.u(body, 8), self.u(body + 8, 8)))
                out.append((mtype, body, msize))
                p = body + msize
        return out

    def heap_name(self, heap_addr, off):
        b = self.b
        if b[heap_addr:heap_addr + 4] != b"HEAP":
            raise H5Error("bad local heap")
        data = self.u(heap_addr + 24, 8)
        end = b.index(b"\0", data + off)
        return b[data + off:end].decode()

    def group_children(self, btree, heap):
        out = []
        b = self.b
        if b[btree:btree + 4] != b"TREE":
            raise H5Error("bad B-tree node")
        level = b[btree + 5]
        used = self.u(btree + 6, 2)
        p = btree + 24
        for i in range(used):
            child = self.u(p + 8, 8)
            p += 16
            if level > 0:
                out += self.group_children(child, heap)
            else:
                if b[child:child + 4] != b"SNOD":
                    raise H5Error("bad symbol node")
                nsym = self.u(child + 6, 2)
                for k in range(nsym):
                    e = self._symbol_entry(child + 8 + 40 * k)
                    out.append((self.heap_name(heap, e["name_off"]), e["header"]))
        return out

    # ---- message decoders ----
    def dataspace(self, off):
        ver = self.b[off]
        ndim = self.b[off + 1]
        if ver == 1:
            p = off + 8
        elif ver == 2:
            p = off + 4
        else:
            raise H5Error(f"dataspace version {ver}")
        return tuple(self.u(p + 8 * i, 8) for i in range(ndim))

    def datatype(self, off):
        cv = self.b[off]
        cls, ver = cv & 0x0F, cv >> 4
        size = self.u(off + 4, 4)
        if cls == 1:  # floating point
            if size == 4:
                return np.dtype("<f4"), 8 + 12
            if size == 8:
                return np.dtype("<f8"), 8 + 12
            raise H5Error("float size")
        if cls == 0:  # fixed point
            signed = bool(self.b[off + 1] & 0x08)
            return np.dtype(("<i" if signed else "<u") + str(size)), 8 + 4
        if cls == 10:  # array
            ndim = self.b[off + 8]
            if ver == 2:
                dims = [self.u(off + 12 + 4 * i, 4) for i in range(ndim)]
                p = off + 12 + 8 * ndim
            else:
                dims = [self.u(off + 9 + 4 * i, 4) for i in range(ndim)]
                p = off + 9 + 4 * ndim
            base, blen = self.datatype(p)
            return np.dtype((base, tuple(dims))), (p - off) + blen
        raise H5Error(f"datatype class {cls}")

    def layout(self, off):
        ver = self.b[off]
        if ver == 3:
            cls = self.b[off + 1]
            if cls == 1:
                return ("contiguous", self.u(off + 2, 8), self.u(off + 10, 8))
            if cls == 0:
                n = self.u(off + 2, 2)
                return ("compact", off + 4, n)
            raise H5Error("chunked layout not supported")
        if ver in (1, 2):
            ndim = self.b[off + 1]
            cls = self.b[off + 2]
            p = off + 8
            if cls == 1:
                addr = self.u(p, 8)
                return ("contiguous", addr, None)
            raise H5Error("layout v1/v2 class")
        raise H5Error(f"layout version {ver}")

    def attribute(self, off):
        ver = self.b[off]
        nlen = self.u(off + 2, 2)
        tlen = self.u(off + 4, 2)
        slen = self.u(off + 6, 2)
        pad = (lambda x: (x + 7) & ~7) if ver == 1 else (lambda x: x)
        p = off + (8 if ver in (1, 2) else 9)
        name = self.b[p:p + nlen].split(b"\0")[0].decode()
        p += pad(nlen)
        dt, _ = self.datatype(p)
        p += pad(tlen)
        shape = self.dataspace(p)
        p += pad(slen)
        count = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(self.b, dtype=dt, count=count, offset=p)
        return name, arr.reshape(shape + dt.shape) if shape else arr

    def node(self, addr):
        msgs = self.messages(addr)
        info = {"attrs": {}}
        for mtype, body, size in msgs:
            if mtype == 0x11:
                info["group"] = (self.u(body, 8), self.u(body + 8, 8))
            elif mtype == 0x01:
                info["shape"] = self.dataspace(body)
            elif mtype == 0x03:
                info["dtype"] = self.datatype(body)[0]
            elif mtype == 0x08:
                info["layout"] = self.layout(body)
            elif mtype == 0x0C:
                k, v = self.attribute(body)
                info["attrs"][k] = v
        return info


class Node:
    def __init__(self, reader: _Reader, addr: int, path: str):
        self._r = reader
        self._info = reader.node(addr)
        self.path = path
        self.attrs = self._info["attrs"]

    @property
    def is_group(self) -> bool:
        return "group" in self._info

    def keys(self):
        bt, heap = self._info["group"]
        return [n for n, _ in self._r.group_children(bt, heap)]

    def __getitem__(self, key: str) -> "Node":
        node = self
        for part in [p for p in key.split("/") if p]:
            bt, heap = node._info["group"]
            kids = dict(node._r.group_children(bt, heap))
            if part not in kids:
                raise KeyError(f"{node.path}/{part}")
            node = Node(node._r, kids[part], node.path.rstrip("/") + "/" + part)
        return node

    def __contains__(self, key: str) -> bool:
        try:
            self[key]
            return True
        except KeyError:
            return False

    def read(self) -> np.ndarray:
        info = self._info
        dt, shape = info["dtype"], info["shape"]
        count = int(np.prod(shape)) if shape else 1
        kind, a, _ = info["layout"]
        if kind == "contiguous" and a == 0xFFFFFFFFFFFFFFFF:
            return np.zeros(shape + dt.shape, dt.base)
        arr = np.frombuffer(self._r.b, dtype=dt, count=count, offset=a)
        return np.array(arr.reshape(shape + dt.shape))


def open_file(path: str) -> Node:
    with open(path, "rb") as f:
        data = f.read()
    r = _Reader(data)
    return Node(r, r.root["header"], "/")


def read_correlations(path: str, group: str):
    """All measurements of `group` (e.g. 'SU2CorZZ') sorted by measurement index:
    (cutoffs[n], data[n, n_basis, n_range])."""
    f = open_file(path)
    g = f[group + "/data"]
    names = sorted(g.keys(), key=lambda x: int(x.split("_")[1]))
    cut = np.array([float(g[n].attrs["cutoff"].reshape(-1)[0]) for n in names], np.float32)
    data = np.stack([g[n + "/data"].read() for n in names])
    return cut, data


def walk(path: str) -> dict:
    """Every object of a file: {"/a/b": {"kind": "group"|"dataset", "attrs": {...},
    "data": array (datasets only)}}."""
    out = {}

    def rec(node: Node, p: str):
        entry = {"kind": "group" if node.is_group else "dataset",
                 "attrs": {k: np.array(v) for k, v in node.attrs.items()}}
        if node.is_group:
            out[p] = entry
            for k in node.keys():
                rec(node[k], p.rstrip("/") + "/" + k)
        else:
            entry["data"] = node.read()
            out[p] = entry

    rec(open_file(path), "/")
    return out


def skeleton(path: str) -> list:
    """Structure without values: [path, kind, sorted attribute names, shape] per object."""
    return [[p, e["kind"], sorted(e["attrs"]), list(e["data"].shape) if "data" in e else None]
            for p, e in sorted(walk(path).items())]


def compare(path_a: str, path_b: str, tolerance: float = 1e-5) -> None:
    """Recursive comparison of two files with the rules of the reference's test evaluator
    (test/scripted/assets/test_eval.py: same members and attributes, max abs deviation below
    the tolerance); raises AssertionError on the first difference."""
    a, b = walk(path_a), walk(path_b)
    assert sorted(a) == sorted(b), f"members differ: {sorted(set(a) ^ set(b))[:10]}"
    for p in a:
        ea, eb = a[p], b[p]
        assert ea["kind"] == eb["kind"], p
        assert sorted(ea["attrs"]) == sorted(eb["attrs"]), f"attributes differ in {p}"
        for k in ea["attrs"]:
            eps = float(np.max(np.abs(ea["attrs"][k] - eb["attrs"][k])))
            assert eps < tolerance, f"deviation in attribute {p}/{k}: {eps}"
        if "data" in ea:
            assert ea["data"].shape == eb["data"].shape, p
            eps = float(np.max(np.abs(ea["data"] - eb["data"]))) if ea["data"].size else 0.0
            assert eps < tolerance, f"deviation in dataset {p}: {eps}"


def layout_fingerprint(path: str) -> dict:
    """Encoding choices of a file, independent of its values: superblock versions and B-tree
    K values, and per object kind the set of header messages with the bytes that encode
    datatypes, fill values, layout classes and dataspace / attribute headers.  Continuation
    and NIL messages (how a writer grew a header) are left out."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    kinds: dict[str, set] = {}

    def key(mtype, body, size):
        raw = r.b[body:body + size]
        if mtype in (0x03, 0x05):
            return raw.hex()
        if mtype == 0x08:
            return raw[:2].hex()
        if mtype == 0x01:
            return raw[:3].hex()
        if mtype == 0x0C:
            nlen = r.u(body + 2, 2)
            tlen = r.u(body + 4, 2)
            p = body + 8 + ((nlen + 7) & ~7)
            return raw[:2].hex() + ":" + r.b[p:p + tlen].hex()
        if mtype == 0x12:
            return raw[:1].hex()
        return ""

    def rec(addr):
        msgs = [(t, key(t, b, s)) for t, b, s in r.messages(addr) if t not in (0x00, 0x10)]
        info = r.node(addr)
        if "group" in info:
            kind = "group"
        else:
            kind = "dataset_" + ("array" if info["dtype"].shape else "scalar")
        kinds.setdefault(kind, set()).update(f"{t:#06x}:{k}" for t, k in msgs)
        if "group" in info:
            for _, child in r.group_children(*info["group"]):
                rec(child)

    rec(r.root["header"])
    return {"superblock": r.b[8:24].hex(), "objects": {k: sorted(v) for k, v in sorted(kinds.items())}}
