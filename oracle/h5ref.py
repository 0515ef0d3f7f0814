"""A pure-Python HDF5 reader and writer: the checker of the library's HDF5
files (test infrastructure; the library never imports it).

Neither machine this project runs on has libhdf5 or h5py, so the library's
reader and writer (test_particle_gb300/csrc/h5lite.cpp) are checked against
this second, independent implementation of the same part of the published
HDF5 file format specification, and this one is pinned to a file libhdf5
itself wrote: scipy's MATLAB 7.3 test file testhdf5_7.4_GLNX86.mat (HDF5 with
a 512-byte user block), whose dataset `testdouble` equals the same variable
scipy reads from the version 5 file testdouble_7.4_GLNX86.mat.

Reader: superblock 0/1, version 1 object headers with continuation blocks,
symbol-table groups (B-tree version 1, symbol-table nodes, local heap),
dataspace 1/2, fixed-point / floating-point / compound datatypes 1-3, layout
messages 1-3 (compact, contiguous, chunked with a version 1 B-tree, no
filters).  `read(path, "/group/dataset")` gives a numpy array in the file's
byte order (structured for compounds).

Writer (`write`): files of the same format with options that make the
variants the library's reader must take (a user block, superblock 1, layout
messages 2 and 3, compact and chunked storage with missing chunks and a fill
value, multi-level chunk B-trees, continuation blocks, dataspace 2, compound
datatypes 1, 2 and 3, nested groups).  Its layout differs from the library
writer's on purpose: data first, then metadata, each dataset's object header
followed by its messages' blocks.
"""
import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(Exception):
    pass


# ------------------------------------------------------------------ reader

def _u(buf, off, n):
    return int.from_bytes(buf[off:off + n], "little")


def _cstr(buf, off):
    end = buf.index(b"\0", off)
    return buf[off:end].decode("latin-1"), end + 1


def _dtype(b, off):
    """Parse one datatype encoding at b[off:]; returns (numpy dtype or None, next offset)."""
    cv = b[off]
    cls, ver = cv & 0x0F, cv >> 4
    bits = _u(b, off + 1, 3)
    size = _u(b, off + 4, 4)
    p = off + 8
    order = ">" if bits & 1 else "<"
    if cls == 0:
        boff, prec = _u(b, p, 2), _u(b, p + 2, 2)
        ok = boff == 0 and prec == 8 * size and size in (1, 2, 4, 8)
        return (np.dtype("%s%s%d" % (order, "i" if bits & 8 else "u", size)) if ok else None), p + 4
    if cls == 1:
        boff, prec = _u(b, p, 2), _u(b, p + 2, 2)
        eloc, esz, mloc, msz, bias = b[p + 4], b[p + 5], b[p + 6], b[p + 7], _u(b, p + 8, 4)
        ieee = {(4, 32, 23, 8, 0, 23, 127), (8, 64, 52, 11, 0, 52, 1023)}
        ok = boff == 0 and not bits & 0x40 and (size, prec, eloc, esz, mloc, msz, bias) in ieee
        return (np.dtype("%sf%d" % (order, size)) if ok else None), p + 12
    if cls == 6:
        n = bits & 0xFFFF
        names, formats, offsets = [], [], []
        supported = True
        obytes = max(1, (size.bit_length() + 7) // 8)
        for _ in range(n):
            name, q = _cstr(b, p)
            if ver < 3:
                q = p + ((q - p + 7) // 8) * 8
                moff = _u(b, q, 4)
                q += 4
                if ver == 1:
                    if b[q] != 0:
                        supported = False
                    q += 28
            else:
                moff = _u(b, q, obytes)
                q += obytes
            mt, p = _dtype(b, q)
            if mt is None:
                supported = False
                continue
            names.append(name)
            formats.append(mt)
            offsets.append(moff)
        if not supported:
            return None, p
        return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size}), p
    raise H5Error("datatype class %d is outside this reader" % cls)


class File:
    def __init__(self, path):
        with open(path, "rb") as fh:
            self.b = fh.read()
        at = 0
        while self.b[at:at + 8] != SIG:
            at = 512 if at == 0 else 2 * at
            if at + 8 > len(self.b):
                raise H5Error("no superblock")
        ver = self.b[at + 8]
        if ver > 1:
            raise H5Error("superblock version %d" % ver)
        if self.b[at + 13] != 8 or self.b[at + 14] != 8:
            raise H5Error("offset/length sizes")
        p = at + 24 + (4 if ver == 1 else 0)
        self.base, _fsi, self.eof, _drv = struct.unpack_from("<4Q", self.b, p)
        self.root = struct.unpack_from("<Q", self.b, p + 40)[0]

    def _a(self, addr):
        return self.base + addr

    def messages(self, oh):
        a = self._a(oh)
        if self.b[a] != 1:
            raise H5Error("object header version %d" % self.b[a])
        nmsg = _u(self.b, a + 2, 2)
        blocks = [(a + 16, _u(self.b, a + 8, 4))]
        out = []
        i = 0
        while i < len(blocks) and len(out) < nmsg:
            start, length = blocks[i]
            q = start
            while q + 8 <= start + length and len(out) < nmsg:
                t, sz, fl = _u(self.b, q, 2), _u(self.b, q + 2, 2), self.b[q + 4]
                body = self.b[q + 8:q + 8 + sz]
                if t == 0x10:
                    blocks.append((self._a(_u(body, 0, 8)), _u(body, 8, 8)))
                out.append((t, fl, body))
                q += 8 + sz
            i += 1
        return out

    def _group_children(self, oh):
        for t, _fl, body in self.messages(oh):
            if t == 0x11:
                bt, hp = _u(body, 0, 8), _u(body, 8, 8)
                h = self._a(hp)
                if self.b[h:h + 4] != b"HEAP":
                    raise H5Error("local heap")
                hdata = self._a(_u(self.b, h + 24, 8))
                return dict(self._btree_group(bt, hdata))
        raise H5Error("not a group")

    def _btree_group(self, node, hdata):
        a = self._a(node)
        if self.b[a:a + 4] != b"TREE" or self.b[a + 4] != 0:
            raise H5Error("group B-tree")
        level, used = self.b[a + 5], _u(self.b, a + 6, 2)
        for i in range(used):
            child = _u(self.b, a + 24 + 8 + 16 * i, 8)
            if level > 0:
                yield from self._btree_group(child, hdata)
                continue
            s = self._a(child)
            if self.b[s:s + 4] != b"SNOD":
                raise H5Error("symbol table node")
            for e in range(_u(self.b, s + 6, 2)):
                en = s + 8 + 40 * e
                name, _ = _cstr(self.b, hdata + _u(self.b, en, 8))
                yield name, _u(self.b, en + 8, 8)

    def lookup(self, path):
        oh = self.root
        for part in [x for x in path.split("/") if x]:
            kids = self._group_children(oh)
            if part not in kids:
                raise H5Error("no object named %r" % part)
            oh = kids[part]
        return oh

    def info(self, path):
        dims, dt, layout, fill, filtered = None, None, None, None, False
        for t, _fl, body in self.messages(self.lookup(path)):
            if t == 0x01:
                ver, rank = body[0], body[1]
                p = 8 if ver == 1 else 4
                dims = [_u(body, p + 8 * d, 8) for d in range(rank)]
            elif t == 0x03:
                dt, _ = _dtype(body, 0)
            elif t == 0x05:
                ver = body[0]
                if ver in (1, 2) and (ver == 1 or body[3]):
                    sz = _u(body, 4, 4)
                    fill = body[8:8 + sz] if sz else None
                elif ver == 3 and body[1] & 0x20:
                    sz = _u(body, 2, 4)
                    fill = body[6:6 + sz]
            elif t == 0x0B:
                filtered = self._filters(body)
            elif t == 0x08:
                layout = self._layout(body)
        if dims is None or layout is None:
            raise H5Error("%s is not a dataset" % path)
        return dims, dt, layout, fill, filtered

    @staticmethod
    def _filters(body):
        ver, n = body[0], body[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = _u(body, p, 2)
            p += 2
            namelen = 0
            if ver == 1 or fid >= 256:
                namelen = _u(body, p, 2)
                p += 2
            p += 2  # flags
            ncd = _u(body, p, 2)
            p += 2
            p += ((namelen + 7) // 8) * 8 if ver == 1 else namelen
            cd = [_u(body, p + 4 * i, 4) for i in range(ncd)]
            p += 4 * ncd + (4 if ver == 1 and ncd % 2 else 0)
            out.append((fid, cd))
        return out

    @staticmethod
    def _unfilter(raw, filters, mask, itemsize):
        import zlib
        for i in range(len(filters) - 1, -1, -1):
            if mask >> i & 1:
                continue
            fid, cd = filters[i]
            if fid == 1:
                raw = zlib.decompress(raw)
            elif fid == 2:
                es = cd[0] if cd else itemsize
                ne = len(raw) // es
                raw = np.frombuffer(raw[:ne * es], np.uint8).reshape(es, ne).T.tobytes() + raw[ne * es:]
            elif fid == 3:
                raw = raw[:-4]
            else:
                raise H5Error("filter %d" % fid)
        return raw

    @staticmethod
    def _layout(body):
        ver = body[0]
        if ver in (1, 2):
            nd, cls = body[1], body[2]
            p = 8
            addr = None
            if cls != 0:
                addr = _u(body, p, 8)
                p += 8
            ld = [_u(body, p + 4 * d, 4) for d in range(nd)]
            p += 4 * nd
            if cls == 0:
                sz = _u(body, p, 4)
                return ("compact", body[p + 4:p + 4 + sz])
            if cls == 1:
                return ("contiguous", addr)
            return ("chunked", addr, ld[:-1])
        if ver == 3:
            cls = body[1]
            if cls == 0:
                sz = _u(body, 2, 2)
                return ("compact", body[4:4 + sz])
            if cls == 1:
                return ("contiguous", _u(body, 2, 8))
            nd = body[2]
            return ("chunked", _u(body, 3, 8), [_u(body, 11 + 4 * d, 4) for d in range(nd - 1)])
        raise H5Error("layout version %d" % ver)

    def read(self, path):
        dims, dt, layout, fill, filtered = self.info(path)
        if dt is None:
            raise H5Error("unsupported datatype")
        n = int(np.prod(dims)) if dims else 1
        shape = tuple(dims)
        if layout[0] == "compact":
            return np.frombuffer(layout[1], dtype=dt, count=n).reshape(shape).copy()
        if layout[0] == "contiguous":
            if layout[1] == UNDEF:
                return self._filled(shape, dt, fill)
            a = self._a(layout[1])
            return np.frombuffer(self.b, dtype=dt, count=n, offset=a).reshape(shape).copy()
        out = self._filled(shape, dt, fill)
        cdims = layout[2]
        n_c = int(np.prod(cdims))
        if layout[1] != UNDEF:
            for offs, addr, size, mask in self._btree_chunks(layout[1], len(dims), bool(filtered)):
                raw = self.b[self._a(addr):self._a(addr) + (size if filtered else n_c * dt.itemsize)]
                if filtered:
                    raw = self._unfilter(raw, filtered, mask, dt.itemsize)
                chunk = np.frombuffer(raw, dtype=dt, count=n_c).reshape(cdims)
                dst = tuple(slice(o, min(o + c, d)) for o, c, d in zip(offs, cdims, dims))
                src = tuple(slice(0, s.stop - s.start) for s in dst)
                out[dst] = chunk[src]
        return out

    @staticmethod
    def _filled(shape, dt, fill):
        out = np.zeros(shape, dtype=dt)
        if fill is not None and len(fill) == dt.itemsize:
            out[...] = np.frombuffer(fill, dtype=dt)[0]
        return out

    def _btree_chunks(self, node, rank, filtered=False):
        a = self._a(node)
        if self.b[a:a + 4] != b"TREE" or self.b[a + 4] != 1:
            raise H5Error("chunk B-tree")
        level, used = self.b[a + 5], _u(self.b, a + 6, 2)
        ks = 8 + 8 * (rank + 1)
        for i in range(used):
            k = a + 24 + i * (ks + 8)
            child = _u(self.b, k + ks, 8)
            if level > 0:
                yield from self._btree_chunks(child, rank, filtered)
            else:
                mask = _u(self.b, k + 4, 4)
                if mask and not filtered:
                    raise H5Error("filtered chunk")
                yield [_u(self.b, k + 8 + 8 * d, 8) for d in range(rank)], child, _u(self.b, k, 4), mask


def read(path, dset):
    return File(path).read(dset)


# ------------------------------------------------------------------ writer

def _enc_atomic(dt):
    dt = np.dtype(dt)
    be = 1 if dt.byteorder == ">" or (dt.byteorder == "=" and np.little_endian is False) else 0
    if dt.kind == "f":
        if dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        else:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        return bytes([0x11, be | 0x20, 8 * dt.itemsize - 1, 0]) + struct.pack("<I", dt.itemsize) + props
    if dt.kind in "iu":
        sgn = 8 if dt.kind == "i" else 0
        return bytes([0x10, be | sgn, 0, 0]) + struct.pack("<I", dt.itemsize) + struct.pack("<HH", 0, 8 * dt.itemsize)
    raise ValueError(dt)


def _enc_type(dt, compound_version=1):
    dt = np.dtype(dt)
    if dt.names is None:
        return _enc_atomic(dt)
    v = compound_version
    out = bytes([(v << 4) | 6]) + len(dt.names).to_bytes(3, "little") + struct.pack("<I", dt.itemsize)
    obytes = max(1, (dt.itemsize.bit_length() + 7) // 8)
    for name in dt.names:
        fdt, off = dt.fields[name][:2]
        nm = name.encode() + b"\0"
        if v < 3:
            nm += b"\0" * (-len(nm) % 8)
            out += nm + struct.pack("<I", off)
            if v == 1:
                out += b"\0" * 28
        else:
            out += nm + off.to_bytes(obytes, "little")
        out += _enc_atomic(fdt)
    return out


class _Out:
    def __init__(self, base):
        self.b = bytearray(base)

    def alloc(self, n, align=8):
        pad = -len(self.b) % align
        self.b += b"\0" * pad
        a = len(self.b)
        self.b += b"\0" * n
        return a

    def put(self, a, data):
        self.b[a:a + len(data)] = data


def _msg(t, body, flags=0):
    body = bytes(body) + b"\0" * (-len(body) % 8)
    return struct.pack("<HHB3x", t, len(body), flags) + body


def write(path, tree, *, userblock=0, superblock=0, layout="contiguous", layout_version=3, chunks=None,
          drop_chunks=(), fill=None, split_header=False, dataspace_version=1, compound_version=1,
          chunk_leaf_entries=64, filters=(), unfiltered_chunks=()):
    """Write `tree` ({name: ndarray or nested dict}) as an HDF5 file; addresses
    are relative to the user block's end (the base address)."""
    o = _Out(b"")
    ub = userblock
    sb_size = 96 + (4 if superblock == 1 else 0)
    o.alloc(ub + sb_size, 1)

    def rel(a):
        return a - ub

    def dataset(arr, name_path):
        arr = np.asarray(arr)
        dt = arr.dtype
        msgs = []
        rank = arr.ndim
        if dataspace_version == 1:
            sp = bytes([1, rank, 0, 0]) + b"\0" * 4 + b"".join(struct.pack("<Q", d) for d in arr.shape)
        else:
            sp = bytes([2, rank, 0, 1 if rank else 0]) + b"".join(struct.pack("<Q", d) for d in arr.shape)
        msgs.append(_msg(0x01, sp))
        msgs.append(_msg(0x03, _enc_type(dt, compound_version), 1))
        if fill is not None:
            fv = np.asarray(fill, dtype=dt).tobytes()
            msgs.append(_msg(0x05, bytes([2, 2, 2, 1]) + struct.pack("<I", len(fv)) + fv, 1))
        raw = np.ascontiguousarray(arr).tobytes()
        lay = layout
        if lay == "chunked" and isinstance(chunks, dict) and name_path not in chunks:
            lay = "contiguous"  # datasets without a chunk shape stay contiguous
        if lay == "compact":
            if layout_version == 3:
                lm = bytes([3, 0]) + struct.pack("<H", len(raw)) + raw
            else:
                lm = bytes([layout_version, rank + 1, 0]) + b"\0" * 5
                lm += b"".join(struct.pack("<I", d) for d in arr.shape) + struct.pack("<I", dt.itemsize)
                lm += struct.pack("<I", len(raw)) + raw
        elif lay == "contiguous":
            addr = rel(o.alloc(len(raw), 16)) if raw else UNDEF
            if raw:
                o.put(addr + ub, raw)
            if layout_version == 3:
                lm = bytes([3, 1]) + struct.pack("<QQ", addr, len(raw))
            else:
                lm = bytes([layout_version, rank + 1, 1]) + b"\0" * 5 + struct.pack("<Q", addr)
                lm += b"".join(struct.pack("<I", d) for d in arr.shape) + struct.pack("<I", dt.itemsize)
        else:
            cd = list(chunks[name_path] if isinstance(chunks, dict) else chunks)
            bt = _write_chunks(o, ub, arr, cd, drop_chunks, chunk_leaf_entries, filters, unfiltered_chunks)
            if filters:
                msgs.append(_msg(0x0B, _pipeline(filters, dt.itemsize), 1))
            if layout_version == 3:
                lm = bytes([3, 2, rank + 1]) + struct.pack("<Q", bt)
            else:
                lm = bytes([layout_version, rank + 1, 2]) + b"\0" * 5 + struct.pack("<Q", bt)
            lm += b"".join(struct.pack("<I", d) for d in cd) + struct.pack("<I", dt.itemsize)
        msgs.append(_msg(0x08, lm))
        return _object_header(o, ub, msgs, split_header)

    def group(node, prefix):
        entries = []
        for name in sorted(node):
            child = node[name]
            if isinstance(child, dict):
                oh, bt, hp = group(child, prefix + "/" + name)
                entries.append((name, oh, (bt, hp)))
            else:
                entries.append((name, dataset(child, (prefix + "/" + name).lstrip("/")), None))
        # local heap: "" at 0, the names, a free block
        data = bytearray(8)
        offs = []
        for name, _, _ in entries:
            offs.append(len(data))
            nm = name.encode() + b"\0"
            data += nm + b"\0" * (-len(nm) % 8)
        free_at = len(data)
        data += struct.pack("<QQ", 1, 16)
        hdata = o.alloc(len(data))
        o.put(hdata, bytes(data))
        heap = o.alloc(32)
        o.put(heap, b"HEAP" + b"\0" * 4 + struct.pack("<QQQ", len(data), free_at, rel(hdata)))
        snods = []
        for s0 in range(0, max(len(entries), 1), 8):
            part = entries[s0:s0 + 8]
            if not part:
                break
            sn = o.alloc(8 + 8 * 40)
            o.put(sn, b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(part)))
            for e, (name, oh, cache) in enumerate(part):
                ent = struct.pack("<QQ", offs[s0 + e], oh)
                if cache:  # a group: cache type 1 with its B-tree and heap
                    ent += struct.pack("<II", 1, 0) + struct.pack("<QQ", *cache)
                else:
                    ent += struct.pack("<II", 0, 0) + b"\0" * 16
                o.put(sn + 8 + 40 * e, ent)
            snods.append((rel(sn), offs[s0 + len(part) - 1]))
        tree = o.alloc(24 + 33 * 8 + 32 * 8)
        node_b = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(snods), UNDEF, UNDEF) + struct.pack("<Q", 0)
        for sn, last in snods:
            node_b += struct.pack("<QQ", sn, last)
        o.put(tree, node_b)
        oh = _object_header(o, ub, [_msg(0x11, struct.pack("<QQ", rel(tree), rel(heap)), 1)], False)
        return oh, rel(tree), rel(heap)

    root_oh, root_bt, root_hp = group(tree, "")
    eof = len(o.b) - ub
    sb = SIG + bytes([superblock, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
    if superblock == 1:
        sb += struct.pack("<HH", 32, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII", 0, root_oh, 1, 0) + struct.pack("<QQ", root_bt, root_hp)
    o.put(ub, sb)
    if ub:
        o.put(0, b"user block".ljust(ub, b"\0"))
    # the superblock's base address is the absolute address of the superblock
    o.put(ub + 24 + (4 if superblock == 1 else 0), struct.pack("<Q", ub))
    with open(path, "wb") as fh:
        fh.write(bytes(o.b))


def _object_header(o, ub, msgs, split):
    if split and len(msgs) > 1:
        rest = b"".join(msgs[1:])
        blk = o.alloc(len(rest))
        o.put(blk, rest)
        first = msgs[0] + _msg(0x10, struct.pack("<QQ", blk - ub, len(rest)))
        n = len(msgs) + 1
    else:
        first = b"".join(msgs)
        n = len(msgs)
    a = o.alloc(16 + len(first))
    o.put(a, bytes([1, 0]) + struct.pack("<HII", n, 1, len(first)) + b"\0" * 4 + first)
    return a - ub


_FILTER_IDS = {"deflate": 1, "shuffle": 2, "fletcher32": 3}


def _pipeline(filters, itemsize):
    """Filter pipeline message version 1 (names padded to 8, client data
    padded to an even count)."""
    out = bytes([1, len(filters)]) + b"\0" * 6
    for name in filters:
        cd = {"deflate": [6], "shuffle": [itemsize], "fletcher32": []}[name]
        nm = name.encode() + b"\0"
        nm += b"\0" * (-len(nm) % 8)
        out += struct.pack("<HHHH", _FILTER_IDS[name], len(nm), 1 if name == "deflate" else 0, len(cd)) + nm
        out += b"".join(struct.pack("<I", v) for v in cd) + (b"\0" * 4 if len(cd) % 2 else b"")
    return out


def _apply_filters(raw, filters, itemsize, mask):
    import zlib
    for i, name in enumerate(filters):
        if mask >> i & 1:
            continue
        if name == "shuffle":
            ne = len(raw) // itemsize
            raw = np.frombuffer(raw[:ne * itemsize], np.uint8).reshape(ne, itemsize).T.tobytes() + raw[ne * itemsize:]
        elif name == "deflate":
            raw = zlib.compress(raw, 6)
        elif name == "fletcher32":
            raw = raw + b"\0\0\0\0"  # the reader strips the checksum without checking it
    return raw


def _write_chunks(o, ub, arr, cd, drop, leaf_entries, filters=(), unfiltered=()):
    """Chunks of arr (edge chunks stored whole, padded with zeros), through
    the filters in order (a chunk listed in `unfiltered` skips them all, as
    its filter mask says), and a version 1 B-tree over them: leaves of up to
    leaf_entries chunks under one level-1 node when there are more."""
    rank = arr.ndim
    grid = [-(-s // c) for s, c in zip(arr.shape, cd)]
    recs = []
    for idx in np.ndindex(*grid):
        if idx in drop:
            continue
        lo = [i * c for i, c in zip(idx, cd)]
        block = np.zeros(cd, dtype=arr.dtype)
        sl = tuple(slice(lo_, min(lo_ + c, s)) for lo_, c, s in zip(lo, cd, arr.shape))
        block[tuple(slice(0, x.stop - x.start) for x in sl)] = arr[sl]
        mask = (1 << len(filters)) - 1 if idx in unfiltered else 0
        raw = _apply_filters(block.tobytes(), filters, arr.dtype.itemsize, mask)
        a = o.alloc(len(raw), 16)
        o.put(a, raw)
        recs.append((lo, a - ub, len(raw), mask))
    ks = 8 + 8 * (rank + 1)

    def key(lo, size, mask=0):
        return struct.pack("<II", size, mask) + b"".join(struct.pack("<Q", x) for x in lo) + struct.pack("<Q", 0)

    def node(level, items, right_key):
        body = b"TREE" + bytes([1, level]) + struct.pack("<HQQ", len(items), UNDEF, UNDEF)
        for k, child in items:
            body += k + struct.pack("<Q", child)
        body += right_key
        a = o.alloc(24 + 129 * ks + 128 * 8)
        o.put(a, body)
        return a - ub

    end_key = key([s for s in arr.shape], 0)
    leaves = []
    for s0 in range(0, len(recs), leaf_entries):
        part = recs[s0:s0 + leaf_entries]
        leaves.append((key(part[0][0], part[0][2], part[0][3]),
                       node(0, [(key(lo, sz, m), a) for lo, a, sz, m in part], end_key)))
    if not leaves:
        return node(0, [], end_key)
    if len(leaves) == 1:
        return leaves[0][1]
    return node(1, leaves, end_key)
