"""A minimal read-only HDF5 walker, enough for the small CGNS/HDF5 mesh files shipped with the
reference's calibration cases: superblock v2/v3, version-2 object headers with continuation
blocks, compact link messages, attribute messages, and datasets with compact or contiguous
layout.  Used only by make_golden.py to turn those files into test fixtures.

Format facts follow the public HDF5 File Format Specification (version 3.0).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


class H5:
    def __init__(self, path: str):
        self.b = open(path, "rb").read()
        b = self.b
        if b[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        ver = b[8]
        if ver not in (2, 3):
            raise ValueError(f"superblock version {ver} not supported")
        self.so, self.sl = b[9], b[10]
        p = 12
        self.base = self._u(p, self.so); p += self.so
        p += self.so  # superblock extension
        p += self.so  # end of file
        self.root = self._u(p, self.so)

    def _u(self, p: int, n: int) -> int:
        return int.from_bytes(self.b[p:p + n], "little")

    # -- object headers ------------------------------------------------------------------
    def messages(self, addr: int):
        b = self.b
        if b[addr:addr + 4] != b"OHDR":
            raise ValueError(f"version-1 object header at {addr} not supported")
        flags = b[addr + 5]
        p = addr + 6
        if flags & 0x20:
            p += 16
        if flags & 0x10:
            p += 4
        csize = 1 << (flags & 3)
        size0 = self._u(p, csize); p += csize
        chunks = [(p, p + size0)]
        out = []
        track_order = bool(flags & 0x04)
        while chunks:
            start, end = chunks.pop(0)
            q = start
            while q + 4 <= end - 4 or (q + 4 <= end and end - q >= 4):
                mtype = b[q]; msize = self._u(q + 1, 2); q += 4
                if track_order:
                    q += 2
                if q + msize > end:
                    break
                data = b[q:q + msize]
                if mtype == 0x10:  # continuation
                    caddr = int.from_bytes(data[:self.so], "little")
                    clen = int.from_bytes(data[self.so:self.so + self.sl], "little")
                    if b[caddr:caddr + 4] == b"OCHK":
                        chunks.append((caddr + 4, caddr + clen - 4))
                elif mtype != 0:
                    out.append((mtype, data))
                q += msize
                if end - q < 4:
                    break
        return out

    def links(self, addr: int) -> dict:
        res = {}
        for t, d in self.messages(addr):
            if t != 0x06:
                continue
            flags = d[1]
            p = 2
            ltype = 0
            if flags & 0x08:
                ltype = d[p]; p += 1
            if flags & 0x04:
                p += 8
            if flags & 0x10:
                p += 1
            ln = 1 << (flags & 3)
            nlen = int.from_bytes(d[p:p + ln], "little"); p += ln
            name = d[p:p + nlen].decode(errors="replace"); p += nlen
            if ltype == 0:
                res[name] = int.from_bytes(d[p:p + self.so], "little")
        return res

    def attrs(self, addr: int) -> dict:
        res = {}
        for t, d in self.messages(addr):
            if t != 0x0C:
                continue
            ver = d[0]
            if ver == 1:
                nsz, tsz, ssz = struct.unpack_from("<HHH", d, 2)
                p = 8
                name = d[p:p + nsz].split(b"\0")[0].decode(); p += (nsz + 7) // 8 * 8
                dt = d[p:p + tsz]; p += (tsz + 7) // 8 * 8
                p += (ssz + 7) // 8 * 8
            else:
                nsz, tsz, ssz = struct.unpack_from("<HHH", d, 2)
                p = 8 + (1 if ver == 3 else 0)
                name = d[p:p + nsz].split(b"\0")[0].decode(); p += nsz
                dt = d[p:p + tsz]; p += tsz
                p += ssz
            size = struct.unpack_from("<I", dt, 4)[0]
            raw = d[p:]
            if (dt[0] & 0x0F) == 3:  # string
                res[name] = raw.split(b"\0")[0].decode(errors="replace")
            else:
                res[name] = raw[:size]
        return res

    def _chunks(self, addr: int, rank: int, out: list):
        """Walk a version-1 B-tree of raw-data chunks (node type 1)."""
        b = self.b
        if b[addr:addr + 4] != b"TREE":
            raise ValueError("bad chunk B-tree")
        level = b[addr + 5]
        used = self._u(addr + 6, 2)
        p = addr + 8 + 2 * self.so
        keysize = 8 + 8 * (rank + 1)
        for i in range(used):
            csize = self._u(p, 4)
            fmask = self._u(p + 4, 4)
            offs = [self._u(p + 8 + 8 * k, 8) for k in range(rank)]
            child = self._u(p + keysize, self.so)
            if level == 0:
                out.append((offs, child, csize, fmask))
            else:
                self._chunks(child, rank, out)
            p += keysize + self.so

    def dataset(self, addr: int) -> np.ndarray:
        dims, dtype, layout = None, None, None
        filters = []
        for t, d in self.messages(addr):
            if t == 0x0B:
                ver, nf = d[0], d[1]
                p = 8 if ver == 1 else 2
                for _ in range(nf):
                    fid = struct.unpack_from("<H", d, p)[0]
                    if ver == 1 or fid >= 256:
                        nlen = struct.unpack_from("<H", d, p + 2)[0]
                        p += 2
                    else:
                        nlen = 0
                    nvals = struct.unpack_from("<H", d, p + 4)[0]
                    p += 6 + ((nlen + 7) // 8 * 8 if ver == 1 else nlen)
                    p += 4 * nvals + (4 if (ver == 1 and nvals % 2) else 0)
                    filters.append(fid)
        for t, d in self.messages(addr):
            if t == 0x01:
                ver, rank, flags = d[0], d[1], d[2]
                p = 8 if ver == 1 else 4
                dims = [int.from_bytes(d[p + i * self.sl:p + (i + 1) * self.sl], "little") for i in range(rank)]
            elif t == 0x03:
                cls = d[0] & 0x0F
                size = struct.unpack_from("<I", d, 4)[0]
                if cls == 0:
                    signed = bool(d[1] & 0x08)
                    dtype = np.dtype(("<i" if signed else "<u") + str(size))
                elif cls == 1:
                    dtype = np.dtype("<f" + str(size))
                elif cls == 3:
                    dtype = np.dtype("S" + str(size))
                else:
                    raise ValueError(f"datatype class {cls} not supported")
            elif t == 0x08:
                ver = d[0]
                if ver < 3:
                    raise ValueError("old layout message")
                cls = d[1]
                if cls == 0:
                    n = struct.unpack_from("<H", d, 2)[0]
                    layout = ("raw", d[4:4 + n])
                elif cls == 1:
                    a = int.from_bytes(d[2:2 + self.so], "little")
                    n = int.from_bytes(d[2 + self.so:2 + self.so + self.sl], "little")
                    layout = ("raw", self.b[a:a + n])
                elif cls == 2:
                    rank = d[2] - 1
                    baddr = int.from_bytes(d[3:3 + self.so], "little")
                    cdims = [struct.unpack_from("<I", d, 3 + self.so + 4 * k)[0] for k in range(rank)]
                    layout = ("chunked", baddr, cdims)
                else:
                    raise ValueError("virtual datasets not supported")
        count = int(np.prod(dims)) if dims else 1
        if layout[0] == "chunked":
            _, baddr, cdims = layout
            full = np.zeros(dims, dtype=dtype)
            chunks = []
            self._chunks(baddr, len(dims), chunks)
            for offs, caddr, csize, fmask in chunks:
                raw = self.b[caddr:caddr + csize]
                for k, fid in reversed(list(enumerate(filters))):
                    if fmask & (1 << k):
                        continue
                    if fid == 1:
                        raw = zlib.decompress(raw)
                    elif fid == 2:
                        n = len(raw) // dtype.itemsize
                        raw = np.frombuffer(raw, np.uint8).reshape(dtype.itemsize, n).T.tobytes()
                    else:
                        raise ValueError(f"filter {fid} not supported")
                blk = np.frombuffer(raw, dtype=dtype, count=int(np.prod(cdims))).reshape(cdims)
                sl = tuple(slice(o, min(o + c, n)) for o, c, n in zip(offs, cdims, dims))
                full[sl] = blk[tuple(slice(0, s.stop - s.start) for s in sl)]
            return full
        arr = np.frombuffer(layout[1], dtype=dtype, count=count)
        # HDF5 stores C order; CGNS writes Fortran arrays with reversed dimensions
        return arr.reshape(dims) if dims else arr

    # -- CGNS helpers ----------------------------------------------------------------------
    def node(self, path):
        addr = self.root
        for name in path:
            addr = self.links(addr)[name]
        return addr

    def cgns_data(self, path) -> np.ndarray:
        return self.dataset(self.links(self.node(path))[" data"])

    def tree(self, addr=None, depth=0, maxdepth=6, out=None):
        out = [] if out is None else out
        addr = self.root if addr is None else addr
        for name, child in sorted(self.links(addr).items()):
            a = {}
            try:
                a = self.attrs(child)
            except ValueError:
                pass
            out.append("  " * depth + f"{name!r} label={a.get('label', '')!r} type={a.get('type', '')!r}")
            if depth < maxdepth and name != " data":
                try:
                    self.tree(child, depth + 1, maxdepth, out)
                except ValueError:
                    pass
        return out
