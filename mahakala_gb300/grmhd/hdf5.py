"""HDF5 reading and writing without h5py, for AthenaK ``.athdf`` snapshots.

The reference loads snapshots with h5py (mahakala/grmhd/athenak.py:77-97):
the datasets ``x1v x2v x3v x1f x2f x3f uov B LogicalLocations Levels`` and
the root attribute ``VariableNames``.  h5py is not available everywhere
this package runs, so this module reads that subset of the HDF5 file format
itself, written from the HDF5 File Format Specification (version 3.0):

* superblock versions 0-3 (a user block before it is allowed: the
  signature is searched at 0, 512, 1024, ...);
* object headers version 1 and 2, with continuation blocks;
* groups stored as a symbol table (version 1 B-tree + local heap + symbol
  nodes, what h5py and the HDF5 library write by default) or as compact
  link messages; dense link storage (fractal heap) is refused with an
  error naming it;
* datasets of fixed-point, floating-point and fixed-length string types in
  either byte order, with compact, contiguous or chunked (version 1 B-tree
  index) layouts; chunk filters deflate, shuffle and Fletcher-32;
* attributes (message versions 1-3) of the same types.

``write_athdf`` writes the same subset (superblock 0, one symbol-table root
group, contiguous datasets -- or uov and B in one chunk per meshblock,
optionally deflated -- and the ``VariableNames`` attribute), so synthetic
snapshots can be stored as files and read back through the reference's
path-based call.
"""

import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
MAX_BLOCKS = 4096     # continuation blocks of one object header
MAX_DEPTH = 64        # B-tree levels


class HDF5Error(ValueError):
    """The file is not HDF5, or uses a part of the format this reader does
    not implement."""


def _align8(n):
    return (n + 7) & ~7


class _Reader:
    def __init__(self, data):
        self.b = data
        self.base = self._find_superblock()
        self._superblock()

    # ------------------------------------------------------------ primitives
    def _find_superblock(self):
        off = 0
        while off + 8 <= len(self.b):
            if self.b[off:off + 8] == SIGNATURE:
                return off
            off = 512 if off == 0 else off * 2
        raise HDF5Error("no HDF5 signature")

    def u(self, at, n):
        if at < 0 or at + n > len(self.b):
            raise HDF5Error(f"read of {n} bytes at {at} outside the file ({len(self.b)} bytes)")
        return int.from_bytes(self.b[at:at + n], "little")

    def addr(self, at):
        return self.u(at, self.so)

    def length(self, at):
        return self.u(at, self.sl)

    def absolute(self, a):
        return self.base_addr + a

    # ------------------------------------------------------------ superblock
    def _superblock(self):
        at = self.base
        ver = self.b[at + 8]
        if ver in (0, 1):
            self.so, self.sl = self.b[at + 13], self.b[at + 14]
            p = at + 24
            if ver == 1:
                p += 4
            self.base_addr = self.addr(p)
            p += 4 * self.so  # base, free-space info, end of file, driver info
            # root group symbol table entry: link name offset, object header address, ...
            self.root = self.addr(p + self.so)
        elif ver in (2, 3):
            self.so, self.sl = self.b[at + 9], self.b[at + 10]
            p = at + 12
            self.base_addr = self.addr(p)
            self.root = self.addr(p + 3 * self.so)
        else:
            raise HDF5Error(f"superblock version {ver} not supported")
        if self.base_addr == UNDEF:
            self.base_addr = 0

    # -------------------------------------------------------- object headers
    def messages(self, oh):
        """(type, data offset, size, flags) of every message of the object
        header at address oh, continuation blocks included."""
        at = self.absolute(oh)
        out = []
        if self.b[at:at + 4] == b"OHDR":
            flags = self.b[at + 5]
            p = at + 6
            if flags & 0x20:
                p += 16
            if flags & 0x10:
                p += 4
            n = 1 << (flags & 3)
            size0 = self.u(p, n)
            p += n
            blocks = [(p, size0, True)]
            seen = 0
            while blocks:
                seen += 1
                if seen > MAX_BLOCKS:
                    raise HDF5Error("object header continuation blocks do not end")
                start, size, first = blocks.pop(0)
                q = start if first else start + 4  # "OCHK"
                end = start + size if first else start + size - 4
                while q + 4 <= end:
                    mtype, msize, mflags = self.b[q], self.u(q + 1, 2), self.b[q + 3]
                    q += 4 + (2 if flags & 0x04 else 0)
                    if mtype == 0x10:
                        blocks.append((self.absolute(self.addr(q)), self.length(q + self.so), False))
                    elif mtype:
                        out.append((mtype, q, msize, mflags))
                    q += msize
            return out
        if self.b[at] != 1:
            raise HDF5Error(f"object header version {self.b[at]} not supported")
        nmsg = self.u(at + 2, 2)
        blocks = [(at + 16, self.u(at + 8, 4))]
        seen = 0
        while blocks and len(out) < nmsg:
            seen += 1
            if seen > MAX_BLOCKS:
                raise HDF5Error("object header continuation blocks do not end")
            start, size = blocks.pop(0)
            q, end = start, start + size
            while q + 8 <= end:
                mtype, msize, mflags = self.u(q, 2), self.u(q + 2, 2), self.b[q + 4]
                q += 8
                if mtype == 0x10:
                    blocks.append((self.absolute(self.addr(q)), self.length(q + self.so)))
                elif mtype:
                    out.append((mtype, q, msize, mflags))
                q += msize
        return out

    # ---------------------------------------------------------------- groups
    def children(self, oh):
        """{name: object header address} of the group at oh."""
        out = {}
        for mtype, p, size, _ in self.messages(oh):
            if mtype == 0x11:  # symbol table
                self._btree_group(self.addr(p), self.addr(p + self.so), out)
            elif mtype == 0x06:  # link
                name, target = self._link(p)
                if target is not None:
                    out[name] = target
            elif mtype == 0x02:  # link info
                flags = self.b[p + 1]
                q = p + 2 + (8 if flags & 1 else 0)
                if self.addr(q) != UNDEF:
                    raise HDF5Error("dense link storage (fractal heap) is not supported")
        return out

    def _heap_data(self, heap):
        at = self.absolute(heap)
        if self.b[at:at + 4] != b"HEAP":
            raise HDF5Error("bad local heap")
        return self.absolute(self.addr(at + 8 + 2 * self.sl))

    def _cstr(self, at):
        end = self.b.find(b"\0", at)
        if at < 0 or end < 0:
            raise HDF5Error("unterminated name in a local heap")
        return self.b[at:end].decode("utf-8")

    def _btree_group(self, tree, heap, out, depth=0):
        if depth > MAX_DEPTH:
            raise HDF5Error("group B-tree deeper than the format allows")
        data = self._heap_data(heap)
        at = self.absolute(tree)
        if self.b[at:at + 4] != b"TREE" or self.b[at + 4] != 0:
            raise HDF5Error("bad group B-tree")
        level, used = self.b[at + 5], self.u(at + 6, 2)
        p = at + 8 + 2 * self.so + self.sl  # first key
        for _ in range(used):
            child = self.addr(p)
            if level > 0:
                self._btree_group(child, heap, out, depth + 1)
            else:
                self._snod(child, data, out)
            p += self.so + self.sl

    def _snod(self, snod, heap_data, out):
        at = self.absolute(snod)
        if self.b[at:at + 4] != b"SNOD":
            raise HDF5Error("bad symbol table node")
        n = self.u(at + 6, 2)
        p = at + 8
        for _ in range(n):
            name = self._cstr(heap_data + self.addr(p))
            out[name] = self.addr(p + self.so)
            p += 2 * self.so + 24

    def _link(self, p):
        flags = self.b[p + 1]
        q = p + 2
        ltype = 0
        if flags & 0x08:
            ltype = self.b[q]
            q += 1
        if flags & 0x04:
            q += 8
        if flags & 0x10:
            q += 1
        nlen_size = 1 << (flags & 3)
        nlen = self.u(q, nlen_size)
        q += nlen_size
        name = self.b[q:q + nlen].decode("utf-8")
        q += nlen
        return name, (self.addr(q) if ltype == 0 else None)

    # --------------------------------------------------------- types, spaces
    def _dtype(self, p):
        cls, ver = self.b[p] & 0x0F, self.b[p] >> 4
        bits = self.b[p + 1]
        size = self.u(p + 4, 4)
        order = ">" if bits & 1 else "<"
        if cls == 0:
            kind = "i" if bits & 0x08 else "u"
            return np.dtype(f"{order}{kind}{size}")
        if cls == 1:
            if size not in (2, 4, 8):
                raise HDF5Error(f"floating-point size {size} not supported")
            return np.dtype(f"{order}f{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise HDF5Error(f"datatype class {cls} (version {ver}) not supported")

    def _dataspace(self, p):
        ver, ndim, flags = self.b[p], self.b[p + 1], self.b[p + 2]
        q = p + (8 if ver == 1 else 4)
        if ver == 2 and self.b[p + 3] == 0:  # scalar
            return ()
        if ver == 2 and self.b[p + 3] == 2:  # null
            return (0,)
        return tuple(self.length(q + i * self.sl) for i in range(ndim))

    # --------------------------------------------------------------- reading
    def dataset(self, oh):
        dtype = shape = layout = None
        filters = []
        for mtype, p, size, _ in self.messages(oh):
            if mtype == 0x01:
                shape = self._dataspace(p)
            elif mtype == 0x03:
                dtype = self._dtype(p)
            elif mtype == 0x08:
                layout = p
            elif mtype == 0x0B:
                filters = self._filters(p)
        if dtype is None or shape is None or layout is None:
            raise HDF5Error("object is not a dataset")
        count = int(np.prod(shape, dtype=np.int64)) if shape else 1
        raw = self._layout_bytes(layout, dtype, shape, count, filters)
        if len(raw) < count * dtype.itemsize:
            raise HDF5Error(f"dataset data truncated ({len(raw)} of {count * dtype.itemsize} bytes)")
        arr = np.frombuffer(raw, dtype=dtype, count=count).reshape(shape)
        return arr.astype(dtype.newbyteorder("=")) if dtype.kind in "iuf" else arr.copy()

    def _filters(self, p):
        ver, n = self.b[p], self.b[p + 1]
        q = p + (8 if ver == 1 else 2)
        out = []
        for _ in range(n):
            fid = self.u(q, 2)
            q += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen = self.u(q, 2)
                q += 2
            q += 2  # flags
            nval = self.u(q, 2)
            q += 2
            q += _align8(nlen) if ver == 1 else nlen
            vals = [self.u(q + 4 * i, 4) for i in range(nval)]
            q += 4 * nval + (4 if ver == 1 and nval % 2 else 0)
            out.append((fid, vals))
        return out

    def _unfilter(self, chunk, filters, mask, itemsize):
        for i in range(len(filters) - 1, -1, -1):
            fid, _ = filters[i]
            if mask >> i & 1:
                continue
            if fid == 1:
                chunk = zlib.decompress(chunk)
            elif fid == 2:
                a = np.frombuffer(chunk, np.uint8)
                n = len(a) // itemsize
                body = a[:n * itemsize].reshape(itemsize, n).T.reshape(-1)
                chunk = body.tobytes() + a[n * itemsize:].tobytes()
            elif fid == 3:
                chunk = chunk[:-4]
            else:
                raise HDF5Error(f"filter {fid} not supported")
        return chunk

    def _layout_bytes(self, p, dtype, shape, count, filters):
        ver = self.b[p]
        nbytes = count * dtype.itemsize
        if ver in (1, 2):
            cls = self.b[p + 2]
            if cls != 1:
                raise HDF5Error(f"layout class {cls} of layout version {ver} not supported")
            a = self.absolute(self.addr(p + 8))
            return self.b[a:a + nbytes]
        if ver not in (3, 4):
            raise HDF5Error(f"layout version {ver} not supported")
        cls = self.b[p + 1]
        if cls == 0:
            size = self.u(p + 2, 2)
            return self.b[p + 4:p + 4 + size]
        if cls == 1:
            a = self.addr(p + 2)
            if a == UNDEF:
                return bytes(nbytes)  # never written: the fill value (zero)
            a = self.absolute(a)
            return self.b[a:a + nbytes]
        if cls == 2 and ver == 3:
            ndim = self.b[p + 2]
            tree = self.addr(p + 3)
            cdims = [self.u(p + 3 + self.so + 4 * i, 4) for i in range(ndim)][:-1]
            out = np.zeros(shape, dtype=dtype)
            if tree != UNDEF:
                self._btree_chunks(tree, len(cdims), cdims, out, filters, dtype)
            return out.tobytes()
        raise HDF5Error(f"layout class {cls} of layout version {ver} not supported")

    def _btree_chunks(self, tree, ndim, cdims, out, filters, dtype, depth=0):
        if depth > MAX_DEPTH:
            raise HDF5Error("chunk B-tree deeper than the format allows")
        at = self.absolute(tree)
        if self.b[at:at + 4] != b"TREE" or self.b[at + 4] != 1:
            raise HDF5Error("bad chunk B-tree")
        level, used = self.b[at + 5], self.u(at + 6, 2)
        ksize = 8 + 8 * (ndim + 1)
        p = at + 8 + 2 * self.so
        for _ in range(used):
            csize, mask = self.u(p, 4), self.u(p + 4, 4)
            offs = [self.u(p + 8 + 8 * i, 8) for i in range(ndim)]
            child = self.addr(p + ksize)
            if level > 0:
                self._btree_chunks(child, ndim, cdims, out, filters, dtype, depth + 1)
            else:
                a = self.absolute(child)
                raw = self._unfilter(self.b[a:a + csize], filters, mask, dtype.itemsize)
                chunk = np.frombuffer(raw, dtype=dtype, count=int(np.prod(cdims))).reshape(cdims)
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, out.shape))
                out[sl] = chunk[tuple(slice(0, s.stop - s.start) for s in sl)]
            p += ksize + self.so

    def attributes(self, oh):
        out = {}
        for mtype, p, size, _ in self.messages(oh):
            if mtype != 0x0C:
                continue
            ver = self.b[p]
            nlen, tlen, slen = self.u(p + 2, 2), self.u(p + 4, 2), self.u(p + 6, 2)
            q = p + 8 + (1 if ver == 3 else 0)
            pad = _align8 if ver == 1 else (lambda n: n)
            name = self.b[q:q + nlen].split(b"\0")[0].decode("utf-8")
            q += pad(nlen)
            dtype = self._dtype(q)
            q += pad(tlen)
            shape = self._dataspace(q)
            q += pad(slen)
            count = int(np.prod(shape, dtype=np.int64)) if shape else 1
            arr = np.frombuffer(self.b[q:q + count * dtype.itemsize], dtype=dtype, count=count).reshape(shape)
            out[name] = arr.astype(dtype.newbyteorder("=")) if dtype.kind in "iuf" else arr.copy()
        return out


def _decoding(fn):
    """Raise HDF5Error for any failure to decode the file (a truncated or
    damaged file surfaces as an index, value, struct or zlib error)."""
    def wrapped(*args, **kwargs):
        try:
            return fn(*args, **kwargs)
        except HDF5Error:
            raise
        except (IndexError, ValueError, struct.error, zlib.error, UnicodeDecodeError, RecursionError) as e:
            raise HDF5Error(f"cannot decode the file: {e}") from e
    wrapped.__name__, wrapped.__doc__ = fn.__name__, fn.__doc__
    return wrapped


class File:
    """A read-only HDF5 file: ``f[name]`` reads a dataset of the root group
    (NumPy array), ``f.attrs`` holds the root group's attributes, ``f.keys()``
    lists the root group's members."""

    @_decoding
    def __init__(self, path):
        with open(path, "rb") as fh:
            self._r = _Reader(fh.read())
        self._members = self._r.children(self._r.root)
        self.attrs = self._r.attributes(self._r.root)

    def keys(self):
        return list(self._members)

    def __contains__(self, name):
        return name in self._members

    def __getitem__(self, name):
        if name not in self._members:
            raise KeyError(name)
        return self._dataset(name)

    @_decoding
    def _dataset(self, name):
        return self._r.dataset(self._members[name])

    @_decoding
    def dataset_attrs(self, name):
        return self._r.attributes(self._members[name])


# ------------------------------------------------------------------ writing
def _dtype_message(dt):
    dt = np.dtype(dt)
    if dt.kind == "S":
        return struct.pack("<BBBBI", 0x13, 0x00, 0, 0, dt.itemsize)  # class 3, version 1, null-terminated ASCII
    order = 1 if dt.byteorder == ">" else 0
    if dt.kind in "iu":
        bits = order | (0x08 if dt.kind == "i" else 0)
        return struct.pack("<BBBBIHH", 0x10, bits, 0, 0, dt.itemsize, 0, 8 * dt.itemsize)
    if dt.kind == "f":
        if dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            sign = 31
        elif dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            sign = 63
        else:
            raise HDF5Error(f"float size {dt.itemsize} not written")
        # bit field: byte order, implied mantissa normalisation (2 << 4), sign position
        return struct.pack("<BBBBI", 0x11, order | 0x20, sign, 0, dt.itemsize) + props
    raise HDF5Error(f"dtype {dt} not written")


def _dataspace_message(shape):
    body = struct.pack("<BBBB4x", 1, len(shape), 0, 0)
    return body + b"".join(struct.pack("<Q", int(n)) for n in shape)


def _message(mtype, body, flags=0):
    body = body + bytes(_align8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(msgs):
    body = b"".join(msgs)
    return struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + bytes(4) + body


def _chunked(put, a, deflate):
    """Raw chunks of a (one chunk per index of its second axis, the
    meshblock axis of uov and B) and the layout and filter messages of a
    chunked dataset with a one-node version 1 B-tree index."""
    if a.ndim < 2 or a.shape[1] > 64:
        raise HDF5Error("chunked writing takes arrays of rank >= 2 with at most 64 blocks")
    cdims = (a.shape[0], 1) + a.shape[2:]
    keys, kids = [], []
    for m in range(a.shape[1]):
        raw = np.ascontiguousarray(a[:, m:m + 1]).tobytes()
        if deflate:
            raw = zlib.compress(raw, 6)
        kids.append(put(raw))
        keys.append(struct.pack("<II", len(raw), 0) + struct.pack(f"<{a.ndim + 1}Q", 0, m, *([0] * (a.ndim - 1))))
    keys.append(struct.pack("<II", 0, 0) + struct.pack(f"<{a.ndim + 1}Q", *a.shape, 0))
    body = b"".join(k + struct.pack("<Q", c) for k, c in zip(keys, kids)) + keys[-1]
    tree = put(b"TREE" + struct.pack("<BBHQQ", 1, 0, a.shape[1], UNDEF, UNDEF) + body)
    layout = struct.pack("<BBBQ", 3, 2, a.ndim + 1, tree) + struct.pack(f"<{a.ndim + 1}I", *cdims, a.itemsize)
    msgs = [_message(0x08, layout)]
    if deflate:
        name = b"deflate\0"
        pipe = (struct.pack("<BB6x", 1, 1) + struct.pack("<HHHH", 1, len(name), 0, 1) + name
                + struct.pack("<I", 6) + bytes(4))
        msgs.append(_message(0x0B, pipe))
    return msgs


def write_athdf(path, arrays, variable_names=None, chunk_blocks=False, deflate=False):
    """Write the datasets and the VariableNames attribute the reference's
    loader reads (athenak.py:77-97) to an HDF5 file at path.  ``arrays`` has
    attributes or keys x1v, x2v, x3v, x1f, x2f, x3f, uov, B,
    LogicalLocations, Levels (a SnapshotArrays works); variable_names
    defaults to arrays.VariableNames.  chunk_blocks stores uov and B in one
    chunk per meshblock (at most 64 blocks), deflate compresses those
    chunks; otherwise every dataset is contiguous."""
    get = (lambda k: arrays[k]) if isinstance(arrays, dict) else (lambda k: getattr(arrays, k))
    names = ["B", "Levels", "LogicalLocations", "uov", "x1f", "x1v", "x2f", "x2v", "x3f", "x3v"]
    data = {k: np.ascontiguousarray(get(k)) for k in names}
    vn = variable_names if variable_names is not None else get("VariableNames")
    width = max(len(v) for v in vn) + 1
    vn_arr = np.array([v.encode("ascii") for v in vn], dtype=f"S{width}")

    out = bytearray()

    def put(b):
        at = len(out)
        out.extend(b)
        out.extend(bytes(_align8(len(out)) - len(out)))
        return at

    # superblock version 0 (fixed size 96 bytes with 8-byte offsets and
    # lengths); filled in at the end
    out.extend(bytes(96))
    # local heap of the root group: "" at offset 0, then the member names
    heap = bytearray(bytes(8))
    name_off = {}
    for k in names:
        name_off[k] = len(heap)
        heap.extend(k.encode("ascii") + b"\0")
        heap.extend(bytes(_align8(len(heap)) - len(heap)))
    # datasets: raw data, then object header (dataspace, datatype, fill value, layout)
    headers = {}
    for k in names:
        a = data[k]
        if chunk_blocks and k in ("uov", "B"):
            store = _chunked(put, a, deflate)
        else:
            store = [_message(0x08, struct.pack("<BBQQ", 3, 1, put(a.tobytes()), a.nbytes))]
        fill = struct.pack("<BBBB", 2, 2, 2, 0)  # version 2, allocation late, written if set, undefined
        headers[k] = put(_object_header([_message(0x01, _dataspace_message(a.shape)),
                                         _message(0x03, _dtype_message(a.dtype), flags=1),
                                         _message(0x05, fill, flags=1)] + store))
    heap_data_at = put(bytes(heap))
    heap_at = put(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), UNDEF, heap_data_at))
    # one symbol table node with every member, sorted by name
    entries = b"".join(struct.pack("<QQII16x", name_off[k], headers[k], 0, 0) for k in sorted(names))
    snod_at = put(b"SNOD" + struct.pack("<BBH", 1, 0, len(names)) + entries)
    # group B-tree: one leaf node, keys "" and the last name
    last = sorted(names)[-1]
    tree_at = put(b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, UNDEF, UNDEF)
                  + struct.pack("<QQQ", 0, snod_at, name_off[last]))
    # root object header: symbol table message and the VariableNames attribute
    aname = b"VariableNames\0"
    adt = _dtype_message(vn_arr.dtype)
    asp = _dataspace_message(vn_arr.shape)
    attr = (struct.pack("<BBHHH", 1, 0, len(aname), len(adt), len(asp))
            + aname + bytes(_align8(len(aname)) - len(aname))
            + adt + bytes(_align8(len(adt)) - len(adt))
            + asp + bytes(_align8(len(asp)) - len(asp)) + vn_arr.tobytes())
    root_at = put(_object_header([_message(0x11, struct.pack("<QQ", tree_at, heap_at)), _message(0x0C, attr)]))
    eof = len(out)
    # group leaf node K = 16 (a symbol node holds up to 32 members), internal K 16
    sb = (SIGNATURE + struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0) + struct.pack("<HHI", 16, 16, 0)
          + struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
          + struct.pack("<QQII", 0, root_at, 1, 0) + struct.pack("<QQ", tree_at, heap_at))
    out[:len(sb)] = sb
    with open(path, "wb") as f:
        f.write(bytes(out))
