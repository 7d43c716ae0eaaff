"""An HDF5 reader and gen_hdf5_write's datasets -- TEST INFRASTRUCTURE ONLY
(tests/ reads the library's HDF5 files with it and compares the datasets
with the restated values).

`read` follows the HDF5 file format specification for the structures a
file of the default (earliest) format holds: superblock versions 0/1, the
root group's symbol table (local heap, version 1 B-tree of group nodes at
any level, symbol table nodes), version 1 object headers with continuation
messages, dataspace versions 1/2, datatypes fixed-point, floating-point,
string and variable-length string (global heap collections), data layout
version 3 (compact and contiguous).  It checks what it walks: signatures,
versions, bounds against the end-of-file address, and alignment of version
1 header messages.  No HDF5 library is available to cross-check it.

`yell` restates gen_hdf5_write (lib_f90/hdf_write.f90:12-326) as the
output menu's 'hdf5' format calls it (discus/prog/graphic.f90:604-635).
Parity unpinned: neither an HDF5 library nor a Fortran compiler is
available to run the reference's writer.
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"


class H5Error(ValueError):
    pass


class _File:
    def __init__(self, b):
        self.b = b
        if b[:8] != SIGNATURE:
            raise H5Error("no HDF5 signature at 0")
        ver = b[8]
        if ver not in (0, 1):
            raise H5Error(f"superblock version {ver}")
        self.so, self.sl = b[13], b[14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("offsets and lengths other than 8 bytes")
        self.leaf_k, self.node_k = struct.unpack_from("<HH", b, 16)
        p = 24 + (4 if ver == 1 else 0)
        self.base, self.freespace, self.eof, self.driver = struct.unpack_from("<4Q", b, p)
        if self.base != 0:
            raise H5Error("base address other than 0")
        if self.eof > len(b):
            raise H5Error(f"end-of-file address {self.eof} beyond the file ({len(b)} bytes)")
        self.root_entry = self.entry(p + 32)

    def need(self, addr, n):
        if addr == UNDEF or addr + n > self.eof:
            raise H5Error(f"{n} bytes at {addr:#x} outside the file")
        return self.b[addr:addr + n]

    def u(self, addr, n):
        return int.from_bytes(self.need(addr, n), "little")

    def entry(self, p):
        name_off, header, cache = struct.unpack_from("<QQI", self.b, p)
        scratch = struct.unpack_from("<QQ", self.b, p + 24)
        return {"name_off": name_off, "header": header, "cache": cache, "scratch": scratch}

    # -------------------------------------------------------- object headers
    def messages(self, addr):
        hdr = self.need(addr, 16)
        if hdr[0] != 1:
            raise H5Error(f"object header version {hdr[0]} at {addr:#x}")
        nmsg = struct.unpack_from("<H", hdr, 2)[0]
        refc, size = struct.unpack_from("<II", hdr, 4)
        chunks = [(addr + 16, size)]
        out = []
        while chunks:
            start, length = chunks.pop(0)
            data = self.need(start, length)
            p = 0
            while p < length:
                if p + 8 > length:
                    raise H5Error("message header past its chunk")
                mtype, msize, flags = struct.unpack_from("<HHB", data, p)
                if msize % 8:
                    raise H5Error(f"message of {msize} bytes not aligned to 8 in a version 1 header")
                body = data[p + 8:p + 8 + msize]
                if len(body) != msize:
                    raise H5Error("message data past its chunk")
                if mtype == 0x10:                       # continuation
                    chunks.append(struct.unpack_from("<QQ", body, 0))
                out.append((mtype, flags, body))
                p += 8 + msize
        if len(out) != nmsg:
            raise H5Error(f"{len(out)} messages, the header says {nmsg}")
        return out

    # -------------------------------------------------------------- groups
    def local_heap(self, addr):
        h = self.need(addr, 32)
        if h[:4] != b"HEAP" or h[4] != 0:
            raise H5Error(f"no version 0 local heap at {addr:#x}")
        size, free, data = struct.unpack_from("<QQQ", h, 8)
        seg = self.need(data, size)
        f = free
        seen = set()
        while f != 1 and f != UNDEF:                      # the free list ends with 1
            if f in seen or f + 16 > size:
                raise H5Error("bad local heap free list")
            seen.add(f)
            f = struct.unpack_from("<Q", seg, f)[0]
        return seg

    @staticmethod
    def name(seg, off):
        end = seg.index(b"\0", off)
        return seg[off:end].decode("ascii")

    def snod(self, addr, seg):
        k2 = 2 * self.leaf_k
        n = self.need(addr, 8 + k2 * 40)
        if n[:4] != b"SNOD" or n[4] != 1:
            raise H5Error(f"no symbol table node at {addr:#x}")
        cnt = struct.unpack_from("<H", n, 6)[0]
        if cnt > k2:
            raise H5Error("symbol table node over its capacity")
        return [(self.name(seg, e["name_off"]), e["header"])
                for e in (self.entry(addr + 8 + 40 * k) for k in range(cnt))]

    def btree(self, addr, seg):
        k2 = 2 * self.node_k
        n = self.need(addr, 24 + k2 * 8 + (k2 + 1) * 8)
        if n[:4] != b"TREE" or n[4] != 0:
            raise H5Error(f"no group B-tree node at {addr:#x}")
        level, used = n[5], struct.unpack_from("<H", n, 6)[0]
        if used > k2:
            raise H5Error("B-tree node over its capacity")
        out = []
        for k in range(used):
            key_lo = struct.unpack_from("<Q", n, 24 + 16 * k)[0]
            child = struct.unpack_from("<Q", n, 32 + 16 * k)[0]
            key_hi = struct.unpack_from("<Q", n, 40 + 16 * k)[0]
            sub = self.snod(child, seg) if level == 0 else self.btree(child, seg)
            lo, hi = self.name(seg, key_lo), self.name(seg, key_hi)
            for nm, _ in sub:
                if not (lo < nm <= hi):
                    raise H5Error(f"name {nm!r} outside its B-tree keys ({lo!r}, {hi!r}]")
            out += sub
        return out

    def group(self, header):
        stab = [b for t, _, b in self.messages(header) if t == 0x11]
        if len(stab) != 1:
            raise H5Error("the root group has no symbol table message")
        tree, heap = struct.unpack_from("<QQ", stab[0], 0)
        entries = self.btree(tree, self.local_heap(heap))
        names = [n for n, _ in entries]
        if names != sorted(names, key=lambda s: s.encode()):
            raise H5Error("symbol table names not in byte order")
        return entries, (tree, heap)

    # ------------------------------------------------------------ datasets
    @staticmethod
    def dataspace(b):
        ver, rank, flags = b[0], b[1], b[2]
        if ver == 1:
            p = 8
        elif ver == 2:
            p = 4
            if b[3] == 2:
                return None                            # null dataspace
        else:
            raise H5Error(f"dataspace version {ver}")
        dims = list(struct.unpack_from(f"<{rank}Q", b, p))
        return tuple(dims)

    def datatype(self, b):
        cls, ver = b[0] & 15, b[0] >> 4
        if ver not in (1, 2, 3):
            raise H5Error(f"datatype version {ver}")
        bf = b[1] | (b[2] << 8) | (b[3] << 16)
        size = struct.unpack_from("<I", b, 4)[0]
        if cls == 0:
            off, prec = struct.unpack_from("<HH", b, 8)
            if off != 0 or prec != 8 * size:
                raise H5Error("fixed-point with padding bits")
            return {"class": "int", "size": size, "order": ">" if bf & 1 else "<", "signed": bool(bf & 8)}
        if cls == 1:
            off, prec, eloc, esz, mloc, msz, bias = struct.unpack_from("<HHBBBBI", b, 8)
            norm, sign = (bf >> 4) & 3, (bf >> 8) & 255
            ieee = {8: (64, 52, 11, 0, 52, 1023, 63), 4: (32, 23, 8, 0, 23, 127, 31)}.get(size)
            if ieee is None or (prec, eloc, esz, mloc, msz, bias, sign) != ieee or off != 0 or norm != 2:
                raise H5Error("floating point other than IEEE binary32/64")
            return {"class": "float", "size": size, "order": ">" if bf & 1 else "<"}
        if cls == 3:
            return {"class": "string", "size": size, "pad": bf & 15, "cset": (bf >> 4) & 15}
        if cls == 9:
            if bf & 15 != 1:
                raise H5Error("variable-length sequences other than strings")
            return {"class": "vlstring", "size": size, "pad": (bf >> 4) & 15, "cset": (bf >> 8) & 15,
                    "base": self.datatype(b[8:])}
        raise H5Error(f"datatype class {cls}")

    def gheap_object(self, addr, index):
        h = self.need(addr, 16)
        if h[:4] != b"GCOL" or h[4] != 1:
            raise H5Error(f"no global heap collection at {addr:#x}")
        size = struct.unpack_from("<Q", h, 8)[0]
        if size < 4096:
            raise H5Error("global heap collection below 4096 bytes")
        col = self.need(addr, size)
        p = 16
        while p + 16 <= size:
            idx, _refs = struct.unpack_from("<HH", col, p)
            osize = struct.unpack_from("<Q", col, p + 8)[0]
            if idx == 0:
                if p + osize != size:
                    raise H5Error("global heap free space does not end the collection")
                break
            if idx == index:
                return col[p + 16:p + 16 + osize]
            p += 16 + ((osize + 7) & ~7)
        raise H5Error(f"global heap object {index} missing")

    def dataset(self, header):
        msgs = self.messages(header)
        by = {}
        for t, _, b in msgs:
            by.setdefault(t, b)
        for t in (0x01, 0x03, 0x08):
            if t not in by:
                raise H5Error(f"dataset without message {t:#x}")
        dims = self.dataspace(by[0x01])
        dt = self.datatype(by[0x03])
        lay = by[0x08]
        if lay[0] != 3:
            raise H5Error(f"layout version {lay[0]}")
        n = int(np.prod(dims)) if dims else 1
        if lay[1] == 0:
            sz = struct.unpack_from("<H", lay, 2)[0]
            raw = lay[4:4 + sz]
        elif lay[1] == 1:
            addr, sz = struct.unpack_from("<QQ", lay, 2)
            raw = self.need(addr, sz) if sz else b""
        else:
            raise H5Error("chunked or virtual layout")
        if len(raw) != n * dt["size"]:
            raise H5Error(f"raw data of {len(raw)} bytes for {n} elements of {dt['size']}")
        if dt["class"] in ("int", "float"):
            kind = "f" if dt["class"] == "float" else ("i" if dt.get("signed") else "u")
            a = np.frombuffer(raw, dtype=np.dtype(f"{dt['order']}{kind}{dt['size']}")).astype(
                np.float64 if kind == "f" else np.int64)
            return a.reshape(dims) if dims else a[0], dt
        if dt["class"] == "string":
            vals = [raw[k * dt["size"]:(k + 1) * dt["size"]] for k in range(n)]
            return (vals if dims else vals[0]), dt
        vals = []
        for k in range(n):
            ln, col, idx = struct.unpack_from("<IQI", raw, 16 * k)
            vals.append(self.gheap_object(col, idx)[:ln])
        return (vals if dims else vals[0]), dt


def read(data):
    """{name: (value, datatype)} for the root group's datasets, plus
    '__file__': the superblock facts."""
    f = _File(bytes(data))
    root = f.root_entry
    entries, (tree, heap) = f.group(root["header"])
    if root["cache"] == 1 and tuple(root["scratch"]) != (tree, heap):
        raise H5Error("the root entry's cached symbol table differs from the group's")
    out = {name: f.dataset(h) for name, h in entries}
    out["__file__"] = {"eof": f.eof, "size": len(data), "leaf_k": f.leaf_k, "node_k": f.node_k}
    return out


def yell(inc, eck, vi, extr, a0, win, value, v, valmax=0.0, scale=1.0):
    """gen_hdf5_write's datasets for qval values v (Fortran order over inc):
    eck (3,4) and vi (3,3) as numpy arrays in the reference's index order."""
    n1, n2, n3 = inc
    q = np.asarray(v, dtype=np.float64).reshape((n1, n2, n3), order="F") * scale     # graphic.f90:618
    vals = np.empty((n1, n2, n3))
    for i in range(n1):                                   # values(k,j,i) = qvalues(i,j,k)
        for j in range(n2):
            for k in range(n3):
                vals[i, j, k] = q[i, j, k]
    if valmax > 0.0:
        finite = vals[~np.isnan(vals)]
        mx = finite.max() if finite.size else np.nan
        if mx >= 0.0:
            vals = (valmax * vals) / mx
    ea, eo, et = extr
    return {
        "data": vals,
        "format": b"Yell 1.0",
        "is_direct": 1 if value in (14, 15) else 0,
        "lower_limits": np.array(eck[:, 0]),
        "step_sizes": np.array([vi[ea - 1, 0], vi[eo - 1, 1], vi[et - 1, 2]]),
        "step_sizes_abs": np.array(vi[:, 0]),
        "step_sizes_ord": np.array(vi[:, 1]),
        "step_sizes_top": np.array(vi[:, 2]),
        "unit_cell": np.array(list(a0) + list(win), dtype=np.float64),
        "PROGRAM": [b"DISCUS60\0"],
    }
