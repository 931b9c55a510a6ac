"""Append-only writer (and a small reader) of netCDF classic files, 64-bit offset format.

The layout is Unidata's published classic format (CDF-2): a header (magic "CDF\\x02",
record count, dimension list, global attributes, variable list with type, padded size
and file offset of each variable), the data of the fixed-size variables, then one
record per step of the unlimited dimension holding every record variable's slab.
Values are big-endian; names, strings and slabs are padded to 4 bytes.

Appending a record writes that record's bytes at the end of the file and rewrites the
4-byte record count in the header, so a frame costs its own bytes only (a writer that
rewrites the whole file at each flush makes a run's output time quadratic in its
frames). Global attributes are written as they are named: a parameter called "mode" is
the attribute "mode".
"""
import struct

import numpy as np

NC_DIMENSION, NC_VARIABLE, NC_ATTRIBUTE = 10, 11, 12
NC_CHAR, NC_INT, NC_DOUBLE = 2, 4, 6
_DTYPE = {NC_INT: ">i4", NC_DOUBLE: ">f8"}
_SIZE = {NC_CHAR: 1, NC_INT: 4, NC_DOUBLE: 8}
_TYPES = {"i4": NC_INT, "f8": NC_DOUBLE}


def _pad4(n):
    return (n + 3) & ~3


def _name(s):
    b = s.encode()
    return struct.pack(">i", len(b)) + b + b"\0" * (_pad4(len(b)) - len(b))


def _attr_value(v):
    """(nc_type, number of elements, padded bytes) of an attribute value: strings as
    NC_CHAR, integers that fit 32 bits as NC_INT, other numbers as NC_DOUBLE."""
    if isinstance(v, bytes):
        v = v.decode()
    if isinstance(v, str):
        b = v.encode()
        return NC_CHAR, len(b), b + b"\0" * (_pad4(len(b)) - len(b))
    if isinstance(v, (bool, np.bool_)):
        v = int(v)
    if isinstance(v, (int, np.integer)) and -2 ** 31 <= int(v) < 2 ** 31:
        return NC_INT, 1, struct.pack(">i", int(v))
    return NC_DOUBLE, 1, struct.pack(">d", float(v))


def _att_list(atts):
    if not atts:
        return struct.pack(">ii", 0, 0)
    out = struct.pack(">ii", NC_ATTRIBUTE, len(atts))
    for k, v in atts.items():
        t, n, data = _attr_value(v)
        out += _name(k) + struct.pack(">ii", t, n) + data
    return out


class ClassicWriter(object):
    """Create `path` and write its header and fixed data; `append` adds records.

    dims: list of (name, size), size None for the unlimited dimension (at most one);
    variables: list of (name, dimension names, "i4" or "f8", attribute dict);
    fixed: {name: array} for every variable that does not run along the unlimited
    dimension. A record variable has the unlimited dimension first."""

    def __init__(self, path, dims, gatts, variables, fixed):
        self.path = path
        self.dims = list(dims)
        self.gatts = dict(gatts)
        dim_index = {d: i for i, (d, _) in enumerate(self.dims)}
        dim_size = dict(self.dims)
        self.vars = []
        for name, vdims, typ, atts in variables:
            t = _TYPES[typ]
            rec = bool(vdims) and dim_size[vdims[0]] is None
            shape = tuple(dim_size[d] for d in vdims[1 if rec else 0:])
            nbytes = int(np.prod(shape, dtype=np.int64)) * _SIZE[t]
            self.vars.append(dict(name=name, dims=[dim_index[d] for d in vdims], type=t, atts=dict(atts), rec=rec,
                                  shape=shape, vsize=_pad4(nbytes), begin=0))
        self.recsize = sum(v["vsize"] for v in self.vars if v["rec"])
        off = len(self._header(0))          # the 8-byte offsets do not change the length
        for v in self.vars:
            if not v["rec"]:
                v["begin"] = off
                off += v["vsize"]
        self.rec_start = off
        for v in self.vars:
            if v["rec"]:
                v["begin"] = off
                off += v["vsize"]
        self.numrecs = 0
        with open(path, "wb") as f:
            f.write(self._header(0))
            for v in self.vars:
                if not v["rec"]:
                    data = np.ascontiguousarray(np.asarray(fixed[v["name"]], dtype=_DTYPE[v["type"]]))
                    if data.shape != v["shape"]:
                        raise ValueError("variable {}: shape {} != {}".format(v["name"], data.shape, v["shape"]))
                    b = data.tobytes()
                    f.write(b + b"\0" * (v["vsize"] - len(b)))

    def _header(self, numrecs):
        out = b"CDF\x02" + struct.pack(">i", numrecs)
        out += struct.pack(">ii", NC_DIMENSION, len(self.dims))
        for name, size in self.dims:
            out += _name(name) + struct.pack(">i", 0 if size is None else size)
        out += _att_list(self.gatts)
        out += struct.pack(">ii", NC_VARIABLE, len(self.vars))
        for v in self.vars:
            out += _name(v["name"]) + struct.pack(">i", len(v["dims"]))
            out += b"".join(struct.pack(">i", d) for d in v["dims"])
            out += _att_list(v["atts"])
            # vsize is 32-bit: a variable of 4 GiB or more records 2^32 - 1
            out += struct.pack(">iIq", v["type"], min(v["vsize"], 0xFFFFFFFF), v["begin"])
        return out

    def append(self, values):
        """Write one record: values[name] for every record variable."""
        with open(self.path, "r+b") as f:
            base = self.numrecs * self.recsize
            for v in self.vars:
                if not v["rec"]:
                    continue
                data = np.ascontiguousarray(np.asarray(values[v["name"]], dtype=_DTYPE[v["type"]]))
                if data.size != max(1, int(np.prod(v["shape"], dtype=np.int64))):
                    raise ValueError("variable {}: {} values for a slab of shape {}".format(
                        v["name"], data.size, v["shape"]))
                b = data.tobytes()
                f.seek(v["begin"] + base)
                f.write(b + b"\0" * (v["vsize"] - len(b)))
            self.numrecs += 1
            f.seek(4)
            f.write(struct.pack(">i", self.numrecs))

    def add_fixed(self, name, vdims, typ, atts, data):
        """Add a variable without the record dimension to an existing file. The header
        grows, so the file is rewritten once with the records it holds."""
        dim_size = dict(self.dims)
        missing = [d for d in vdims if d not in dim_size]
        if missing or any(dim_size[d] is None for d in vdims):
            raise ValueError("variable {}: dimensions {} are not fixed dimensions of {}".format(
                name, list(vdims), self.path))
        if any(v["name"] == name for v in self.vars):
            raise ValueError("variable {} already exists in {}".format(name, self.path))
        _, _, old = read(self.path)
        dim_names = [d for d, _ in self.dims]
        variables, fixed = [], {}
        for v in self.vars:
            typ_v = "i4" if v["type"] == NC_INT else "f8"
            variables.append((v["name"], tuple(dim_names[d] for d in v["dims"]), typ_v, v["atts"]))
            if not v["rec"]:
                fixed[v["name"]] = old[v["name"]][1]
        variables.append((name, tuple(vdims), typ, atts))
        fixed[name] = data
        numrecs = self.numrecs
        self.__init__(self.path, self.dims, self.gatts, variables, fixed)
        for r in range(numrecs):
            self.append({v["name"]: old[v["name"]][1][r] for v in self.vars if v["rec"]})


def read(path):
    """(dimensions, global attributes, {name: (attributes, array)}) of a classic file
    (CDF-1 or CDF-2) with NC_CHAR/NC_INT/NC_DOUBLE attributes and NC_INT/NC_DOUBLE
    variables; record variables come back with the record axis first."""
    with open(path, "rb") as f:
        buf = f.read()
    pos = [0]

    def take(fmt):
        vals = struct.unpack_from(fmt, buf, pos[0])
        pos[0] += struct.calcsize(fmt)
        return vals if len(vals) > 1 else vals[0]

    def name():
        n = take(">i")
        s = buf[pos[0]:pos[0] + n].decode()
        pos[0] += _pad4(n)
        return s

    def atts():
        tag, n = take(">ii")
        out = {}
        for _ in range(n):
            k = name()
            t, cnt = take(">ii")
            raw = buf[pos[0]:pos[0] + cnt * _SIZE[t]]
            pos[0] += _pad4(cnt * _SIZE[t])
            out[k] = raw.decode() if t == NC_CHAR else np.frombuffer(raw, dtype=_DTYPE[t])[0].item()
        return out

    magic = buf[:4]
    if magic not in (b"CDF\x01", b"CDF\x02"):
        raise ValueError("not a netCDF classic file: " + path)
    pos[0] = 4
    numrecs = take(">i")
    _, ndims = take(">ii")
    dims = [(name(), take(">i")) for _ in range(ndims)]
    gatts = atts()
    _, nvars = take(">ii")
    vars_ = []
    for _ in range(nvars):
        vname = name()
        nd = take(">i")
        vd = [take(">i") for _ in range(nd)]
        va = atts()
        t, _ = take(">iI")
        begin = take(">q" if magic == b"CDF\x02" else ">i")
        rec_var = bool(vd) and dims[vd[0]][1] == 0
        slab = [dims[d][1] for d in vd[1 if rec_var else 0:]]
        vars_.append((vname, vd, va, t, _pad4(int(np.prod(slab, dtype=np.int64)) * _SIZE[t]), begin))
    rec = [v for v in vars_ if v[1] and dims[v[1][0]][1] == 0]
    recsize = sum(v[4] for v in rec)
    out = {}
    for vname, vd, va, t, vsize, begin in vars_:
        shape = tuple(dims[d][1] for d in vd)
        if vd and dims[vd[0]][1] == 0:
            slab = shape[1:]
            cnt = int(np.prod(slab, dtype=np.int64))
            arr = np.empty((numrecs,) + slab, dtype=_DTYPE[t])
            for r in range(numrecs):
                arr[r] = np.frombuffer(buf, dtype=_DTYPE[t], count=cnt, offset=begin + r * recsize).reshape(slab)
        else:
            cnt = int(np.prod(shape, dtype=np.int64))
            arr = np.frombuffer(buf, dtype=_DTYPE[t], count=cnt, offset=begin).reshape(shape).copy()
        out[vname] = (va, arr.astype(arr.dtype.newbyteorder("=")))
    return dims, gatts, out
