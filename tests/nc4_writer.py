"""A minimal netCDF-4 (HDF5) writer for the tests of aeroapps_gb300/nc4.py:
root-group float64 variables with named dimensions, laid out as the HDF5 file
format specification describes and as netCDF-4 uses it (superblock 2,
version-2 object headers, compact links, dimension scales, DIMENSION_LIST
references in a global heap), with a choice of chunk index (version-1
B-tree, fixed array, single chunk, implicit) and filters (shuffle, deflate).
Checksum fields are left zero (the reader does not check them).  Test
infrastructure: the package never writes HDF5."""
import zlib

import numpy as np

O = L = 8
UNDEF = (1 << 64) - 1


def _u(v, n):
    return int(v).to_bytes(n, "little")


class _Buf:
    def __init__(self):
        self.b = bytearray()

    def put(self, data, align=8):
        while len(self.b) % align:
            self.b.append(0)
        a = len(self.b)
        self.b += data
        return a


def _f64():
    # floating point, version 1; little-endian, mantissa normalised (implied
    # msb), sign at bit 63; offset 0, precision 64, exponent 52+11 bits, bias 1023
    return bytes([0x11, 0x20, 0x3F, 0x00]) + _u(8, 4) + _u(0, 2) + _u(64, 2) + bytes([52, 11, 0, 52]) + _u(1023, 4)


def _string(n):
    return bytes([0x13, 0x00, 0x00, 0x00]) + _u(n, 4)


_LEGACY = [False]  # superblock 0, version-1 object headers and messages, symbol-table root group


def _pad8(b):
    return b + bytes((-len(b)) % 8)


def _dataspace(shape):
    if _LEGACY[0]:
        return bytes([1, len(shape), 0, 0]) + bytes(4) + b"".join(_u(s, L) for s in shape)
    return bytes([2, len(shape), 0, 1 if shape else 0]) + b"".join(_u(s, L) for s in shape)


def _msg(t, body):
    return (t, body)


def _ohdr(msgs):
    if _LEGACY[0]:
        body = b"".join(_u(t, 2) + _u(len(_pad8(b)), 2) + bytes(4) + _pad8(b) for t, b in msgs)
        return bytes([1, 0]) + _u(len(msgs), 2) + _u(1, 4) + _u(len(body), 4) + bytes(4) + body
    body = b"".join(bytes([t]) + _u(len(b), 2) + b"\0" + b for t, b in msgs)
    return b"OHDR" + bytes([2, 0x02]) + _u(len(body), 4) + body + b"\0\0\0\0"


def _attr(name, dtype, space, data):
    nm = name.encode() + b"\0"
    if _LEGACY[0]:
        return _msg(0x0C, bytes([1, 0]) + _u(len(nm), 2) + _u(len(dtype), 2) + _u(len(space), 2)
                    + _pad8(nm) + _pad8(dtype) + _pad8(space) + data)
    return _msg(0x0C, bytes([3, 0]) + _u(len(nm), 2) + _u(len(dtype), 2) + _u(len(space), 2) + b"\0"
                + nm + dtype + space + data)


def _str_attr(name, s):
    v = s.encode() + b"\0"
    return _attr(name, _string(len(v)), _dataspace(()), v)


def write(path, dims, variables, index="btree1", chunk=None, shuffle=True, deflate=True, legacy=False):
    """dims: [(name, length, coordinate values or None)]; variables:
    [(name, dimension names, float64 array)].  Variables are chunked with
    chunk(shape) -> chunk shape (default: halves, rounded up) through the
    chosen index; coordinate variables are contiguous.  legacy: the layout
    of files from HDF5 1.6-era writers (superblock 0, version-1 object
    headers, a symbol-table root group; version-1 B-tree chunk index only)."""
    assert not legacy or index == "btree1"
    _LEGACY[0] = legacy
    try:
        _write(path, dims, variables, index, chunk, shuffle, deflate, legacy)
    finally:
        _LEGACY[0] = False


def _write(path, dims, variables, index, chunk, shuffle, deflate, legacy):
    buf = _Buf()
    buf.put(bytes(96 if legacy else 48))  # superblock, written last
    filters = []
    # (id, flags, client values); version 2 messages, or version 1 (with a
    # name length field and padding to 8 bytes) in the legacy layout
    for fid, vals in ([(2, [8])] if shuffle else []) + ([(1, [6])] if deflate else []):
        if legacy:
            filters.append(_u(fid, 2) + _u(0, 2) + _u(1, 2) + _u(len(vals), 2) + b"".join(_u(v, 4) for v in vals)
                           + bytes(4 * (len(vals) % 2)))
        else:
            filters.append(_u(fid, 2) + _u(1, 2) + _u(len(vals), 2) + b"".join(_u(v, 4) for v in vals))
    pipeline = (bytes([1, len(filters)]) + bytes(6) if legacy else bytes([2, len(filters)])) + b"".join(filters)
    links, dim_addr = [], {}

    def contiguous(values):
        a = buf.put(np.ascontiguousarray(values, "<f8").tobytes())
        return _msg(0x08, bytes([3, 1]) + _u(a, O) + _u(values.size * 8, L))

    for name, n, coord in dims:
        if coord is None:
            lay = _msg(0x08, bytes([3, 1]) + _u(UNDEF, O) + _u(0, L))
            label = "This is a netCDF dimension but not a netCDF variable. %10d" % n
        else:
            lay = contiguous(np.asarray(coord, np.float64))
            label = name
        a = buf.put(_ohdr([_msg(0x01, _dataspace((n,))), _msg(0x03, _f64()), lay,
                           _str_attr("CLASS", "DIMENSION_SCALE"), _str_attr("NAME", label)]))
        dim_addr[name] = a
        links.append((name, a))
    # DIMENSION_LIST objects: one global heap object (one reference) per dimension
    names = [d[0] for d in dims]
    objs = b""
    for i, name in enumerate(names):
        objs += _u(i + 1, 2) + _u(1, 2) + bytes(4) + _u(O, L) + _u(dim_addr[name], O)
    objs += _u(0, 2) + bytes(6) + _u(0, L)
    gcol = buf.put(b"GCOL" + bytes([1, 0, 0, 0]) + _u(16 + len(objs), L) + objs)
    vlen = bytes([0x19, 0x00, 0x00, 0x00]) + _u(4 + O + 4, 4) + bytes([0x17, 0, 0, 0]) + _u(O, 4)
    for name, vdims, arr in variables:
        arr = np.ascontiguousarray(arr, "<f8")
        shape = arr.shape
        cdims = list(chunk(shape) if chunk else [-(-s // 2) for s in shape])
        grid = [-(-s // c) for s, c in zip(shape, cdims)]
        chunks = []
        for k in range(int(np.prod(grid))):
            offs = [int(x) * c for x, c in zip(np.unravel_index(k, grid), cdims)]
            block = np.zeros(cdims, "<f8")
            src = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
            block[tuple(slice(0, sl.stop - sl.start) for sl in src)] = arr[src]
            raw = block.tobytes()
            if index != "implicit":
                if shuffle:
                    raw = np.frombuffer(raw, np.uint8).reshape(-1, 8).T.tobytes()
                if deflate:
                    raw = zlib.compress(raw, 6)
            chunks.append((offs, raw))
        esize_dims = cdims + [8]
        rank1 = len(esize_dims)
        if index == "btree1":
            addrs = [buf.put(raw) for _, raw in chunks]
            body = b"TREE" + bytes([1, 0]) + _u(len(chunks), 2) + _u(UNDEF, O) + _u(UNDEF, O)
            for (offs, raw), a in zip(chunks, addrs):
                body += _u(len(raw), 4) + _u(0, 4) + b"".join(_u(o, 8) for o in offs + [0]) + _u(a, O)
            body += _u(0, 4) + _u(0, 4) + b"".join(_u(s, 8) for s in list(shape) + [0])
            tree = buf.put(body)
            lay = _msg(0x08, bytes([3, 2, rank1]) + _u(tree, O) + b"".join(_u(x, 4) for x in esize_dims))
        else:
            head = bytes([4, 2])
            if index == "farray":
                addrs = [buf.put(raw) for _, raw in chunks]
                ent = O + 4 + 4
                db = len(buf.b) + (-len(buf.b)) % 8
                hdr_at = db + 4 + 2 + O + ent * len(chunks) + 4
                hdr_at += (-hdr_at) % 8
                buf.put(b"FADB" + bytes([0, 1]) + _u(hdr_at, O)
                        + b"".join(_u(a, O) + _u(len(raw), 4) + _u(0, 4) for a, (_, raw) in zip(addrs, chunks))
                        + bytes(4))
                got = buf.put(b"FAHD" + bytes([0, 1, ent, 10]) + _u(len(chunks), L) + _u(db, O) + bytes(4))
                assert got == hdr_at
                info = bytes([3, 10]) + _u(got, O)
                flags = 0
            elif index == "single":
                assert len(chunks) == 1
                raw = chunks[0][1]
                info = bytes([1]) + _u(len(raw), L) + _u(0, 4) + _u(buf.put(raw), O)
                flags = 0x02
            elif index == "implicit":
                first = None
                for _, raw in chunks:
                    a = buf.put(raw, align=1)
                    first = a if first is None else first
                info = bytes([2]) + _u(first, O)
                flags = 0
            else:
                raise ValueError(index)
            lay = _msg(0x08, head + bytes([flags, rank1, 4]) + b"".join(_u(x, 4) for x in esize_dims) + info)
        refs = b"".join(_u(1, 4) + _u(gcol, O) + _u(names.index(d) + 1, 4) for d in vdims)
        msgs = [_msg(0x01, _dataspace(shape)), _msg(0x03, _f64()), lay]
        if index != "implicit" and (shuffle or deflate):
            msgs.append(_msg(0x0B, pipeline))
        msgs.append(_attr("DIMENSION_LIST", vlen, _dataspace((len(vdims),)), refs))
        links.append((name, buf.put(_ohdr(msgs))))
    if legacy:
        # root group: local heap of link names, one symbol table node, a
        # one-leaf version-1 B-tree; names in ascending order
        links.sort()
        heap, offs = bytearray(bytes(8)), []
        for name, _ in links:
            offs.append(len(heap))
            heap += _pad8(name.encode() + b"\0")
        seg = buf.put(bytes(heap))
        lheap = buf.put(b"HEAP" + bytes(4) + _u(len(heap), L) + _u(UNDEF, L) + _u(seg, O))
        ents = b"".join(_u(o, O) + _u(a, O) + bytes(24) for o, (_, a) in zip(offs, links))
        snod = buf.put(b"SNOD" + bytes([1, 0]) + _u(len(links), 2) + ents)
        tree = buf.put(b"TREE" + bytes([0, 0]) + _u(1, 2) + _u(UNDEF, O) + _u(UNDEF, O)
                       + _u(0, L) + _u(snod, O) + _u(offs[-1], L))
        root = buf.put(_ohdr([_msg(0x11, _u(tree, O) + _u(lheap, O))]))
        buf.b[0:96] = b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, O, L, 0]) + _u(4, 2) + _u(16, 2) + bytes(4) \
            + _u(0, O) + _u(UNDEF, O) + _u(len(buf.b), O) + _u(UNDEF, O) \
            + _u(0, O) + _u(root, O) + _u(1, 4) + bytes(4) + _u(tree, O) + _u(lheap, O)
    else:
        lmsgs = []
        for name, a in links:
            nm = name.encode()
            lmsgs.append(_msg(0x06, bytes([1, 0]) + _u(len(nm), 1) + nm + _u(a, O)))
        root = buf.put(_ohdr(lmsgs))
        buf.b[0:48] = b"\x89HDF\r\n\x1a\n" + bytes([2, O, L, 0]) + _u(0, O) + _u(UNDEF, O) + _u(len(buf.b), O) \
            + _u(root, O) + bytes(4)
    with open(path, "wb") as fh:
        fh.write(bytes(buf.b))
