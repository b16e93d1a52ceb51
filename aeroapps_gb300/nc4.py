"""Read-only access to netCDF-4 files (the HDF5 format) for the Mie optics tables.

GEOS optics tables (optics_*.nc) may be netCDF-4 files, which
Chem_MieTableRead opens through the netCDF library (nf90_open, nf90_inq_dimid,
nf90_get_var: Chem_MieTableMod.F90:297-466).  Neither the netCDF nor the HDF5
library is available to this package, so this module reads the part of the
HDF5 file format (HDF Group, "HDF5 File Format Specification Version 3.0")
that netCDF-4 writes for fixed-size numeric variables in the root group:

- superblocks 0-3; object headers 1 and 2 with their continuation blocks;
- groups held as symbol tables (version-1 B-tree and local heap), as compact
  link messages, or as dense links (fractal heap with a version-2 B-tree name
  index);
- dataspaces, fixed-point and floating-point datatypes of either byte order,
  fill values;
- compact, contiguous and chunked layouts, chunks indexed by a version-1
  B-tree, a single chunk, an implicit list or a fixed array, with the
  deflate, shuffle and Fletcher-32 filters;
- attributes of numbers or strings, and DIMENSION_LIST, the variable-length
  object references (global heap) that name a variable's dimensions.

Any other construct raises ValueError naming it.  The reader parses a file
already in memory and never writes."""
import zlib

import numpy as np

MAGIC = b"\x89HDF\r\n\x1a\n"

# header message types
_DATASPACE, _LINKINFO, _DATATYPE, _FILL_OLD, _FILL, _LINK = 0x1, 0x2, 0x3, 0x4, 0x5, 0x6
_LAYOUT, _FILTERS, _ATTRIBUTE, _CONTINUATION, _SYMTAB = 0x8, 0xB, 0xC, 0x10, 0x11
_ATTRINFO = 0x15

# filter ids
_DEFLATE, _SHUFFLE, _FLETCHER32 = 1, 2, 3


class _Datatype:
    """A decoded datatype message: kind 'num' (numpy dtype), 'str' (fixed
    length), 'ref' (object reference) or 'vlen' (base: another _Datatype)."""

    def __init__(self, kind, size, dtype=None, base=None, vlen_string=False):
        self.kind, self.size, self.dtype, self.base, self.vlen_string = kind, size, dtype, base, vlen_string


class H5File:
    """An HDF5 file held in memory: groups, datasets and attributes by address."""

    def __init__(self, path):
        with open(path, "rb") as fh:
            self.d = fh.read()
        self.path = path
        base = self.d.find(MAGIC)
        if base != 0:
            raise ValueError("%s: no HDF5 signature at the start of the file" % path)
        ver = self.d[8]
        if ver in (0, 1):
            self.O, self.L = self.d[13], self.d[14]
            p = 24 if ver == 0 else 28
            # base, free-space, end-of-file and driver addresses, then the root
            # group's symbol table entry (link name offset, object header address)
            self.root = self._u(p + 5 * self.O, self.O)
        elif ver in (2, 3):
            self.O, self.L = self.d[9], self.d[10]
            self.root = self._u(12 + 3 * self.O, self.O)
        else:
            raise ValueError("%s: HDF5 superblock version %d" % (path, ver))
        self.undef = (1 << (8 * self.O)) - 1

    # ------------------------------------------------------------------ bytes
    def _u(self, off, n):
        return int.from_bytes(self.d[off:off + n], "little")

    def _sig(self, off, sig):
        if self.d[off:off + 4] != sig:
            raise ValueError("%s: expected %s at %d, found %r" % (self.path, sig.decode(), off, self.d[off:off + 4]))

    # ------------------------------------------------------------ object headers
    def messages(self, addr):
        """[(type, offset, size)] of the object header at addr, continuation
        blocks followed."""
        d, out = self.d, []
        if d[addr:addr + 4] == b"OHDR":
            flags = d[addr + 5]
            p = addr + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
            nsz = 1 << (flags & 3)
            size0 = self._u(p, nsz)
            p += nsz
            blocks = [(p, p + size0)]
            hdr = 6 if flags & 0x04 else 4
            while blocks:
                p, end = blocks.pop(0)
                while p + hdr <= end:
                    t, sz = d[p], self._u(p + 1, 2)
                    p += hdr
                    out.append((t, p, sz))
                    if t == _CONTINUATION:
                        ca, cl = self._u(p, self.O), self._u(p + self.O, self.L)
                        self._sig(ca, b"OCHK")
                        blocks.append((ca + 4, ca + cl - 4))  # signature ... checksum
                    p += sz
        elif d[addr] == 1:
            hsz = self._u(addr + 8, 4)
            blocks = [(addr + 16, addr + 16 + hsz)]
            while blocks:
                p, end = blocks.pop(0)
                while p + 8 <= end:
                    t, sz = self._u(p, 2), self._u(p + 2, 2)
                    p += 8
                    out.append((t, p, sz))
                    if t == _CONTINUATION:
                        ca, cl = self._u(p, self.O), self._u(p + self.O, self.L)
                        blocks.append((ca, ca + cl))
                    p += sz
        else:
            raise ValueError("%s: no object header at %d" % (self.path, addr))
        return out

    # ------------------------------------------------------------------ groups
    def links(self, addr):
        """{name: object header address} of the hard links of the group at addr."""
        out = {}
        for t, p, sz in self.messages(addr):
            if t == _LINK:
                name, target = self._link(p)
                if target is not None:
                    out[name] = target
            elif t == _LINKINFO:
                flags = self.d[p + 1]
                q = p + 2 + (8 if flags & 1 else 0)
                heap, names = self._u(q, self.O), self._u(q + self.O, self.O)
                if heap != self.undef:
                    out.update(self._dense_links(heap, names))
            elif t == _SYMTAB:
                out.update(self._symtab_links(self._u(p, self.O), self._u(p + self.O, self.O)))
        return out

    def _link(self, p):
        d = self.d
        if d[p] != 1:
            raise ValueError("%s: link message version %d" % (self.path, d[p]))
        flags = d[p + 1]
        q = p + 2
        ltype = 0
        if flags & 0x08:
            ltype = d[q]
            q += 1
        if flags & 0x04:
            q += 8
        if flags & 0x10:
            q += 1
        nl = 1 << (flags & 3)
        n = self._u(q, nl)
        q += nl
        name = d[q:q + n].decode("utf-8")
        q += n
        return name, (self._u(q, self.O) if ltype == 0 else None)

    def _symtab_links(self, btree, heap):
        self._sig(heap, b"HEAP")
        seg = self._u(heap + 8 + 2 * self.L, self.O)
        out = {}

        def node(addr):
            self._sig(addr, b"TREE")
            level, used = self.d[addr + 5], self._u(addr + 6, 2)
            p = addr + 8 + 2 * self.O + self.L  # past the header and key 0
            for _ in range(used):
                child = self._u(p, self.O)
                p += self.O + self.L
                if level > 0:
                    node(child)
                else:
                    self._sig(child, b"SNOD")
                    q = child + 8
                    for _ in range(self._u(child + 6, 2)):
                        noff, oh = self._u(q, self.O), self._u(q + self.O, self.O)
                        end = self.d.index(b"\0", seg + noff)
                        out[self.d[seg + noff:end].decode("utf-8")] = oh
                        q += 2 * self.O + 24
        node(btree)
        return out

    def _dense_links(self, heap, btree):
        fh = _FractalHeap(self, heap)
        out = {}
        for rec in _btree2_records(self, btree, 5):
            name, target = self._link(fh.object(rec[4:]))
            if target is not None:
                out[name] = target
        return out

    # ----------------------------------------------------------------- datasets
    def dataset(self, addr):
        """Shape, datatype, layout, filters, fill value and attributes of the
        dataset at addr."""
        ds = {"shape": None, "dtype": None, "layout": None, "filters": [], "fill": None, "attrs": {}}
        for t, p, sz in self.messages(addr):
            if t == _DATASPACE:
                ds["shape"] = self._dataspace(p)
            elif t == _DATATYPE:
                ds["dtype"] = self._datatype(p)
            elif t == _LAYOUT:
                ds["layout"] = self._layout(p)
            elif t == _FILTERS:
                ds["filters"] = self._filters(p)
            elif t == _FILL:
                ds["fill"] = self._fill(p)
            elif t == _FILL_OLD and ds["fill"] is None:
                n = self._u(p, 4)
                ds["fill"] = self.d[p + 4:p + 4 + n] if n else None
            elif t == _ATTRIBUTE:
                name, value = self._attribute(p)
                ds["attrs"][name] = value
            elif t == _ATTRINFO:
                flags = self.d[p + 1]
                q = p + 2 + (2 if flags & 1 else 0)
                heap, names = self._u(q, self.O), self._u(q + self.O, self.O)
                if heap != self.undef:
                    fh = _FractalHeap(self, heap)
                    for rec in _btree2_records(self, names, 8):
                        name, value = self._attribute(fh.object(rec[:8]))
                        ds["attrs"][name] = value
        return ds

    def _dataspace(self, p):
        d = self.d
        ver, rank, flags = d[p], d[p + 1], d[p + 2]
        if ver == 1:
            q = p + 8
        elif ver == 2:
            if d[p + 3] == 2:  # null dataspace
                return None
            q = p + 4
        else:
            raise ValueError("%s: dataspace version %d" % (self.path, ver))
        return tuple(self._u(q + self.L * i, self.L) for i in range(rank))

    def _datatype(self, p):
        d = self.d
        cls, bits, size = d[p] & 0x0F, self._u(p + 1, 3), self._u(p + 4, 4)
        order = ">" if bits & 1 else "<"
        if cls == 0:
            dt = np.dtype("%s%s%d" % (order, "i" if bits & 0x08 else "u", size))
            return _Datatype("num", size, dtype=dt)
        if cls == 1:
            if size not in (2, 4, 8):
                raise ValueError("%s: %d-byte floating point" % (self.path, size))
            return _Datatype("num", size, dtype=np.dtype("%sf%d" % (order, size)))
        if cls == 3:
            return _Datatype("str", size)
        if cls == 7:
            return _Datatype("ref", size)
        if cls == 9:
            return _Datatype("vlen", size, base=self._datatype(p + 8), vlen_string=(bits & 0x0F) == 1)
        raise ValueError("%s: datatype class %d" % (self.path, cls))

    def _layout(self, p):
        d = self.d
        ver, cls = d[p], d[p + 1]
        if ver not in (3, 4):
            raise ValueError("%s: data layout version %d" % (self.path, ver))
        if cls == 0:
            n = self._u(p + 2, 2)
            return {"class": "compact", "data": d[p + 4:p + 4 + n]}
        if cls == 1:
            return {"class": "contiguous", "addr": self._u(p + 2, self.O), "size": self._u(p + 2 + self.O, self.L)}
        if cls != 2:
            raise ValueError("%s: data layout class %d" % (self.path, cls))
        if ver == 3:
            rank = d[p + 2]
            addr = self._u(p + 3, self.O)
            q = p + 3 + self.O
            dims = [self._u(q + 4 * i, 4) for i in range(rank)]
            return {"class": "chunked", "index": "btree1", "addr": addr, "chunk": dims[:-1], "esize": dims[-1]}
        flags, rank, enc = d[p + 2], d[p + 3], d[p + 4]
        q = p + 5
        dims = [self._u(q + enc * i, enc) for i in range(rank)]
        q += enc * rank
        itype = d[q]
        q += 1
        lay = {"class": "chunked", "chunk": dims[:-1], "esize": dims[-1]}
        if itype == 1:
            lay["index"] = "single"
            if flags & 0x02:
                lay["fsize"], lay["fmask"] = self._u(q, self.L), self._u(q + self.L, 4)
                q += self.L + 4
        elif itype == 2:
            lay["index"] = "implicit"
        elif itype == 3:
            lay["index"] = "farray"
            q += 1
        else:
            raise ValueError("%s: chunk index type %d (extensible array / v2 B-tree: unlimited dimensions)"
                             % (self.path, itype))
        lay["addr"] = self._u(q, self.O)
        return lay

    def _filters(self, p):
        d = self.d
        ver, n = d[p], d[p + 1]
        q = p + (8 if ver == 1 else 2)
        out = []
        for _ in range(n):
            fid = self._u(q, 2)
            if ver == 1 or fid >= 256:
                nlen = self._u(q + 2, 2)
                flags, nval = self._u(q + 4, 2), self._u(q + 6, 2)
                q += 8
                q += ((nlen + 7) // 8) * 8 if ver == 1 else nlen
            else:
                flags, nval = self._u(q + 2, 2), self._u(q + 4, 2)
                q += 6
            vals = [self._u(q + 4 * i, 4) for i in range(nval)]
            q += 4 * nval
            if ver == 1 and nval % 2:
                q += 4
            out.append((fid, vals))
        return out

    def _fill(self, p):
        d = self.d
        ver = d[p]
        if ver in (1, 2):
            defined = d[p + 3]
            if ver == 1 or defined:
                n = self._u(p + 4, 4)
                return d[p + 8:p + 8 + n] if n else None
            return None
        if ver == 3:
            flags = d[p + 1]
            if flags & 0x20:
                n = self._u(p + 2, 4)
                return d[p + 6:p + 6 + n]
            return None
        raise ValueError("%s: fill value version %d" % (self.path, ver))

    # --------------------------------------------------------------- attributes
    def _attribute(self, p):
        d = self.d
        ver = d[p]
        nlen, tlen, slen = self._u(p + 2, 2), self._u(p + 4, 2), self._u(p + 6, 2)
        if ver == 1:
            pad = lambda n: ((n + 7) // 8) * 8
            q = p + 8
            name = d[q:q + nlen].split(b"\0")[0].decode("utf-8")
            q += pad(nlen)
            tq = q
            q += pad(tlen)
            sq = q
            q += pad(slen)
        elif ver in (2, 3):
            if d[p + 1] & 0x03:
                raise ValueError("%s: shared datatype or dataspace in an attribute" % self.path)
            q = p + 8 + (1 if ver == 3 else 0)
            name = d[q:q + nlen].split(b"\0")[0].decode("utf-8")
            q += nlen
            tq = q
            q += tlen
            sq = q
            q += slen
        else:
            raise ValueError("%s: attribute message version %d" % (self.path, ver))
        try:
            dt = self._datatype(tq)
        except ValueError:  # e.g. the compound REFERENCE_LIST of a dimension scale: not needed here
            return name, None
        shape = self._dataspace(sq)
        return name, self._values(dt, shape, q)

    def _values(self, dt, shape, q):
        if shape is None:
            return None
        n = int(np.prod(shape)) if len(shape) else 1
        if dt.kind == "num":
            a = np.frombuffer(self.d, dt.dtype, n, q).astype(dt.dtype.newbyteorder("="))
            return a.reshape(shape) if len(shape) else a[0]
        if dt.kind == "str":
            vals = [self.d[q + dt.size * i:q + dt.size * (i + 1)].split(b"\0")[0].decode("utf-8", "replace")
                    for i in range(n)]
            return vals[0] if not len(shape) else vals
        if dt.kind == "ref":
            return [self._u(q + dt.size * i, self.O) for i in range(n)]
        # variable length: (length, global heap collection, object index) per element
        vals = []
        for i in range(n):
            e = q + i * (4 + self.O + 4)
            cnt, coll, idx = self._u(e, 4), self._u(e + 4, self.O), self._u(e + 4 + self.O, 4)
            raw = self._global_object(coll, idx) if cnt else b""
            if dt.vlen_string:
                vals.append(raw.split(b"\0")[0].decode("utf-8", "replace"))
            elif dt.base.kind == "ref":
                vals.append([int.from_bytes(raw[self.O * k:self.O * (k + 1)], "little") for k in range(cnt)])
            elif dt.base.kind == "num":
                vals.append(np.frombuffer(raw, dt.base.dtype, cnt).copy())
            else:
                raise ValueError("%s: variable-length attribute of %s" % (self.path, dt.base.kind))
        return vals[0] if not len(shape) else vals

    def _global_object(self, coll, idx):
        self._sig(coll, b"GCOL")
        end = coll + self._u(coll + 8, self.L)
        q = coll + 8 + self.L
        while q + 8 + self.L <= end:
            oi, size = self._u(q, 2), self._u(q + 8, self.L)
            if oi == 0:
                break
            if oi == idx:
                return self.d[q + 8 + self.L:q + 8 + self.L + size]
            q += 8 + self.L + ((size + 7) // 8) * 8
        raise ValueError("%s: global heap object %d not in collection %d" % (self.path, idx, coll))

    # -------------------------------------------------------------------- data
    def read(self, ds):
        """The values of a dataset (from dataset()) as a C-order numpy array."""
        shape, dt, lay = ds["shape"], ds["dtype"], ds["layout"]
        if shape is None:
            return None
        if dt.kind != "num":
            raise ValueError("%s: reading a dataset of %s values" % (self.path, dt.kind))
        n = int(np.prod(shape)) if len(shape) else 1
        if lay["class"] == "compact":
            raw = lay["data"]
        elif lay["class"] == "contiguous":
            if lay["addr"] == self.undef:
                return self._filled(ds, shape)
            raw = self.d[lay["addr"]:lay["addr"] + n * dt.size]
        else:
            return self._chunked(ds)
        a = np.frombuffer(raw, dt.dtype, n)
        return a.astype(dt.dtype.newbyteorder("=")).reshape(shape)

    def _filled(self, ds, shape):
        dt = ds["dtype"]
        fill = np.frombuffer(ds["fill"], dt.dtype, 1)[0] if ds["fill"] else 0
        return np.full(shape, fill, dt.dtype.newbyteorder("="))

    def _chunks(self, ds):
        """[(chunk offsets, file address, stored size, filter mask)]."""
        lay, shape = ds["layout"], ds["shape"]
        cdims, rank = lay["chunk"], len(lay["chunk"])
        full = int(np.prod(cdims)) * lay["esize"]
        grid = [-(-s // c) for s, c in zip(shape, cdims)]
        order = [tuple(int(x) * c for x, c in zip(np.unravel_index(k, grid), cdims))
                 for k in range(int(np.prod(grid)))]
        idx = lay["index"]
        if idx == "btree1":
            out = []

            def node(addr):
                self._sig(addr, b"TREE")
                level, used = self.d[addr + 5], self._u(addr + 6, 2)
                ksz = 8 + 8 * (rank + 1)
                p = addr + 8 + 2 * self.O
                for _ in range(used):
                    size, mask = self._u(p, 4), self._u(p + 4, 4)
                    offs = tuple(self._u(p + 8 + 8 * i, 8) for i in range(rank))
                    child = self._u(p + ksz, self.O)
                    if level > 0:
                        node(child)
                    else:
                        out.append((offs, child, size, mask))
                    p += ksz + self.O
            if lay["addr"] != self.undef:
                node(lay["addr"])
            return out
        if idx == "single":
            return [(order[0], lay["addr"], lay.get("fsize", full), lay.get("fmask", 0))]
        if idx == "implicit":
            return [(o, lay["addr"] + k * full, full, 0) for k, o in enumerate(order)]
        # fixed array
        a = lay["addr"]
        if a == self.undef:
            return []
        self._sig(a, b"FAHD")
        client, esize, pbits = self.d[a + 5], self.d[a + 6], self.d[a + 7]
        nent = self._u(a + 8, self.L)
        db = self._u(a + 8 + self.L, self.O)
        if nent > (1 << pbits):
            raise ValueError("%s: paged fixed-array chunk index (%d chunks)" % (self.path, nent))
        self._sig(db, b"FADB")
        q = db + 6 + self.O
        out = []
        for k in range(nent):
            e = q + k * esize
            addr = self._u(e, self.O)
            if client == 1:
                ssz = esize - self.O - 4
                size, mask = self._u(e + self.O, ssz), self._u(e + self.O + ssz, 4)
            else:
                size, mask = full, 0
            if addr != self.undef:
                out.append((order[k], addr, size, mask))
        return out

    def _chunked(self, ds):
        shape, dt, lay = ds["shape"], ds["dtype"], ds["layout"]
        out = self._filled(ds, shape)
        cdims = lay["chunk"]
        for offs, addr, size, mask in self._chunks(ds):
            raw = self._unfilter(self.d[addr:addr + size], ds["filters"], mask, dt.size)
            c = np.frombuffer(raw, dt.dtype, int(np.prod(cdims))).reshape(cdims)
            dst = tuple(slice(o, min(o + cd, s)) for o, cd, s in zip(offs, cdims, shape))
            src = tuple(slice(0, sl.stop - sl.start) for sl in dst)
            out[dst] = c[src]
        return out

    def _unfilter(self, raw, filters, mask, esize):
        for i in range(len(filters) - 1, -1, -1):
            if mask & (1 << i):
                continue
            fid, vals = filters[i]
            if fid == _DEFLATE:
                raw = zlib.decompress(raw)
            elif fid == _SHUFFLE:
                es = vals[0] if vals else esize
                n = len(raw) // es
                body = np.frombuffer(raw, np.uint8, n * es).reshape(es, n).T.tobytes()
                raw = body + raw[n * es:]
            elif fid == _FLETCHER32:
                raw = raw[:-4]
            else:
                raise ValueError("%s: filter %d" % (self.path, fid))
        return raw


class _FractalHeap:
    """The managed objects of a fractal heap (direct blocks reached from a
    root direct block or a root indirect block of direct blocks)."""

    def __init__(self, f, addr):
        f._sig(addr, b"FRHP")
        self.f = f
        O, L = f.O, f.L
        self.idlen = f._u(addr + 5, 2)
        filt_len = f._u(addr + 7, 2)
        self.flags = f.d[addr + 9]
        q = addr + 14 + L + O + L + O + 8 * L  # past max managed size and the statistics
        self.width = f._u(q, 2)
        self.start = f._u(q + 2, L)
        self.maxdirect = f._u(q + 2 + L, L)
        self.maxheap = f._u(q + 2 + 2 * L, 2)
        self.root = f._u(q + 6 + 2 * L, O)
        self.rows = f._u(q + 6 + 2 * L + O, 2)
        if filt_len:
            raise ValueError("%s: filtered fractal heap" % f.path)
        self.offbytes = (self.maxheap + 7) // 8
        self.blocks = []  # (heap offset, size, file address) of the direct blocks
        if self.rows == 0:
            self.blocks.append((0, self.start, self.root))
        else:
            f._sig(self.root, b"FHIB")
            p = self.root + 5 + O + self.offbytes
            off = 0
            for r in range(self.rows):
                size = self.start * (1 << max(r - 1, 0))
                if size > self.maxdirect:
                    raise ValueError("%s: fractal heap with indirect child blocks" % f.path)
                for _ in range(self.width):
                    a = f._u(p, O)
                    p += O
                    if a != f.undef:
                        self.blocks.append((off, size, a))
                    off += size

    def object(self, hid):
        """File offset of the managed object with heap ID hid."""
        f = self.f
        if (hid[0] >> 4) & 3 != 0:
            raise ValueError("%s: huge or tiny fractal heap object" % f.path)
        off = int.from_bytes(hid[1:1 + self.offbytes], "little")
        n = int.from_bytes(hid[1 + self.offbytes:self.idlen], "little")
        for boff, size, a in self.blocks:
            if boff <= off < boff + size:
                f._sig(a, b"FHDB")
                if off - boff + n > size:
                    raise ValueError("%s: fractal heap object crosses its block" % f.path)
                return a + (off - boff)
        raise ValueError("%s: fractal heap offset %d outside its blocks" % (f.path, off))


def _btree2_records(f, addr, rtype):
    """Records of the version-2 B-tree at addr (leaf root, or one level of
    internal node over leaves)."""
    f._sig(addr, b"BTHD")
    if f.d[addr + 5] != rtype:
        raise ValueError("%s: version-2 B-tree of type %d, expected %d" % (f.path, f.d[addr + 5], rtype))
    node_size, rsize, depth = f._u(addr + 6, 4), f._u(addr + 10, 2), f._u(addr + 12, 2)
    root, nroot = f._u(addr + 16, f.O), f._u(addr + 16 + f.O, 2)

    def leaf(a, n):
        f._sig(a, b"BTLF")
        return [f.d[a + 6 + rsize * i:a + 6 + rsize * (i + 1)] for i in range(n)]

    if depth == 0:
        return leaf(root, nroot) if root != f.undef else []
    if depth > 1:
        raise ValueError("%s: version-2 B-tree of depth %d" % (f.path, depth))
    f._sig(root, b"BTIN")
    maxleaf = (node_size - 10) // rsize
    nb = (maxleaf.bit_length() + 7) // 8
    recs = [f.d[root + 6 + rsize * i:root + 6 + rsize * (i + 1)] for i in range(nroot)]
    p = root + 6 + rsize * nroot
    out = []
    for i in range(nroot + 1):
        child, n = f._u(p, f.O), f._u(p + f.O, nb)
        p += f.O + nb
        out.extend(leaf(child, n))
        if i < nroot:
            out.append(recs[i])
    return out


class Variable:
    """One netCDF-4 variable: its dimension names, shape and attributes;
    values() reads it."""

    def __init__(self, f, name, addr, ds, dims):
        self._f, self.name, self.addr, self._ds = f, name, addr, ds
        self.dimensions, self.shape, self.attributes = dims, ds["shape"], ds["attrs"]

    def values(self):
        return self._f.read(self._ds)


class Dataset:
    """The root group of a netCDF-4 file: dimensions {name: length} and
    variables {name: Variable}, as nf90_inq_dimid / nf90_inq_varid see them."""

    def __init__(self, path):
        f = H5File(path)
        self.path = path
        links = f.links(f.root)
        by_addr = {a: n for n, a in links.items()}
        sets = {}
        for name, addr in links.items():
            ds = f.dataset(addr)
            if ds["layout"] is None:  # a group
                continue
            sets[name] = (addr, ds)
        self.dimensions = {}
        for name, (addr, ds) in sets.items():
            if ds["attrs"].get("CLASS") == "DIMENSION_SCALE":
                self.dimensions[name] = int(ds["shape"][0]) if ds["shape"] else 0
        self.variables = {}
        for name, (addr, ds) in sets.items():
            is_scale = ds["attrs"].get("CLASS") == "DIMENSION_SCALE"
            if is_scale and str(ds["attrs"].get("NAME", "")).startswith("This is a netCDF dimension but not"):
                continue  # a dimension without a coordinate variable
            dl = ds["attrs"].get("DIMENSION_LIST")
            if dl is not None:
                dims = tuple(by_addr[refs[0]] for refs in dl)
            elif is_scale:
                dims = (name,)
            else:
                dims = tuple("dim%d" % i for i in range(len(ds["shape"] or ())))
            self.variables[name] = Variable(f, name, addr, ds, dims)
