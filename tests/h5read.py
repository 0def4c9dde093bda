"""A reader of the HDF5 subset iskra_write_openpmd writes, written from the
published HDF5 file format specification independently of the writer (test
infrastructure: no HDF5 library or h5py exists on these machines).

Reads: the version 2 superblock; version 2 object headers ("OHDR") with
their link info / group info / link (hard, compact storage), dataspace
(version 2), datatype (fixed point, floating point, string), fill value,
data layout (version 3, contiguous) and attribute (version 3) messages.
Every metadata checksum (superblock, object headers) is verified with an
own implementation of Jenkins' lookup3 hashlittle.
"""
import struct

import numpy as np


def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 hashlittle (2006, public domain)."""
    M = 0xFFFFFFFF

    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & M

    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M
    i = 0
    while n - i > 12:
        a = (a + struct.unpack_from("<I", data, i)[0]) & M
        b = (b + struct.unpack_from("<I", data, i + 4)[0]) & M
        c = (c + struct.unpack_from("<I", data, i + 8)[0]) & M
        a = (a - c) & M; a ^= rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 4); b = (b + a) & M
        i += 12
    rest = data[i:]
    if not rest:
        return c
    tail = rest + bytes(12 - len(rest))
    a = (a + struct.unpack_from("<I", tail, 0)[0]) & M
    b = (b + struct.unpack_from("<I", tail, 4)[0]) & M
    c = (c + struct.unpack_from("<I", tail, 8)[0]) & M
    c ^= b; c = (c - rot(b, 14)) & M
    a ^= c; a = (a - rot(c, 11)) & M
    b ^= a; b = (b - rot(a, 25)) & M
    c ^= b; c = (c - rot(b, 16)) & M
    a ^= c; a = (a - rot(c, 4)) & M
    b ^= a; b = (b - rot(a, 14)) & M
    c ^= b; c = (c - rot(b, 24)) & M
    return c


class H5Error(ValueError):
    pass


def _datatype(buf, o):
    """(numpy dtype or ('str', size), byte length) of a datatype message at o."""
    cls_ver = buf[o]
    cls, ver = cls_ver & 0x0F, cls_ver >> 4
    bits = buf[o + 1:o + 4]
    size = struct.unpack_from("<I", buf, o + 4)[0]
    if ver != 1:
        raise H5Error(f"datatype version {ver}")
    if cls == 0:  # fixed point
        signed = bool(bits[0] & 0x08)
        if bits[0] & 0x01:
            raise H5Error("big-endian integer")
        return np.dtype(f"{'<i' if signed else '<u'}{size}"), 12
    if cls == 1:  # floating point: IEEE little-endian only
        if bits[0] & 0x41:
            raise H5Error("unsupported float byte order")
        prec, exp_loc, exp_sz, man_loc, man_sz = struct.unpack_from("<xxHBBBB", buf, o + 8)
        bias = struct.unpack_from("<I", buf, o + 16)[0]
        if size == 8 and (prec, exp_loc, exp_sz, man_loc, man_sz, bias) == (64, 52, 11, 0, 52, 1023):
            return np.dtype("<f8"), 20
        if size == 4 and (prec, exp_loc, exp_sz, man_loc, man_sz, bias) == (32, 23, 8, 0, 23, 127):
            return np.dtype("<f4"), 20
        raise H5Error("non-IEEE float layout")
    if cls == 3:  # string
        return ("str", size), 8
    raise H5Error(f"datatype class {cls}")


def _dataspace(buf, o):
    ver, rank, flags, typ = buf[o], buf[o + 1], buf[o + 2], buf[o + 3]
    if ver != 2:
        raise H5Error(f"dataspace version {ver}")
    dims = list(struct.unpack_from(f"<{rank}Q", buf, o + 4)) if rank else []
    n = 4 + 8 * rank * (2 if flags & 1 else 1)
    return (None if typ == 0 else tuple(dims)), n


def _decode(buf, dt, shape, o):
    count = int(np.prod(shape)) if shape else 1
    if isinstance(dt, tuple):
        raw = bytes(buf[o:o + dt[1] * count])
        vals = [raw[k * dt[1]:(k + 1) * dt[1]].split(b"\0")[0].decode() for k in range(count)]
        return vals[0] if shape is None else vals
    arr = np.frombuffer(bytes(buf[o:o + dt.itemsize * count]), dtype=dt)
    return arr[0] if shape is None else arr.reshape(shape)


class Object:
    def __init__(self, f, addr):
        self.attrs, self.links = {}, {}
        self.shape = self.dtype = self.data_addr = self.data_size = None
        buf = f.buf
        if buf[addr:addr + 4] != b"OHDR":
            raise H5Error(f"no object header at {addr}")
        ver, flags = buf[addr + 4], buf[addr + 5]
        if ver != 2:
            raise H5Error(f"object header version {ver}")
        o = addr + 6
        if flags & 0x20:
            o += 16
        if flags & 0x10:
            o += 4
        szb = 1 << (flags & 3)
        size = int.from_bytes(buf[o:o + szb], "little")
        o += szb
        end = o + size
        if end + 4 > len(buf):
            raise H5Error(f"object header at {addr} runs past the end of the file")
        if lookup3(bytes(buf[addr:end])) != struct.unpack_from("<I", buf, end)[0]:
            raise H5Error(f"object header checksum at {addr}")
        while o + 4 <= end:
            mtype, msize, mflags = buf[o], struct.unpack_from("<H", buf, o + 1)[0], buf[o + 3]
            o += 4
            if flags & 0x04:
                o += 2
            body = o
            if mtype == 0x01:
                self.shape, _ = _dataspace(buf, body)
            elif mtype == 0x03:
                self.dtype, _ = _datatype(buf, body)
            elif mtype == 0x08:
                if buf[body] != 3 or buf[body + 1] != 1:
                    raise H5Error("only contiguous version 3 layouts")
                self.data_addr, self.data_size = struct.unpack_from("<QQ", buf, body + 2)
            elif mtype == 0x06:
                lver, lflags = buf[body], buf[body + 1]
                p = body + 2
                if lver != 1:
                    raise H5Error("link version")
                ltype = 0
                if lflags & 0x08:
                    ltype = buf[p]
                    p += 1
                if lflags & 0x04:
                    p += 8
                if lflags & 0x10:
                    p += 1
                lb = 1 << (lflags & 3)
                nlen = int.from_bytes(buf[p:p + lb], "little")
                p += lb
                name = bytes(buf[p:p + nlen]).decode()
                p += nlen
                if ltype != 0:
                    raise H5Error("only hard links")
                self.links[name] = struct.unpack_from("<Q", buf, p)[0]
            elif mtype == 0x0C:
                aver = buf[body]
                if aver != 3:
                    raise H5Error("attribute version")
                nsz, dsz, ssz = struct.unpack_from("<HHH", buf, body + 2)
                p = body + 9
                name = bytes(buf[p:p + nsz]).split(b"\0")[0].decode()
                p += nsz
                dt, _ = _datatype(buf, p)
                p += dsz
                shape, _ = _dataspace(buf, p)
                p += ssz
                self.attrs[name] = _decode(buf, dt, shape, p)
            o = body + msize

    @property
    def is_dataset(self):
        return self.data_addr is not None


class File:
    def __init__(self, path):
        self.buf = memoryview(open(path, "rb").read())
        buf = self.buf
        if bytes(buf[:8]) != b"\x89HDF\r\n\x1a\n":
            raise H5Error("no HDF5 signature")
        if buf[8] not in (2, 3):
            raise H5Error(f"superblock version {buf[8]}")
        if buf[9] != 8 or buf[10] != 8:
            raise H5Error("only 8-byte offsets and lengths")
        base, ext, eof, root = struct.unpack_from("<QQQQ", buf, 12)
        if lookup3(bytes(buf[:44])) != struct.unpack_from("<I", buf, 44)[0]:
            raise H5Error("superblock checksum")
        if eof != len(buf):
            raise H5Error(f"end of file {eof} != size {len(buf)}")
        self.root = root

    def get(self, path):
        obj = Object(self, self.root)
        for part in [p for p in path.split("/") if p]:
            if part not in obj.links:
                raise KeyError(path)
            obj = Object(self, obj.links[part])
        return obj

    def read(self, path):
        obj = self.get(path)
        if not obj.is_dataset:
            raise H5Error(f"{path} is a group")
        n = int(np.prod(obj.shape))
        if obj.data_size != n * obj.dtype.itemsize:
            raise H5Error("layout size does not match the dataspace")
        return np.frombuffer(bytes(self.buf[obj.data_addr:obj.data_addr + obj.data_size]),
                             dtype=obj.dtype).reshape(obj.shape)
