"""Writer of the reference's k-space file layout (MRI_DATA::write_external_data, the
HDF5 C++ library's defaults as src/hdf5_interface.cpp uses them) for the tests of the
library's HDF5 reader -- test infrastructure, no HDF5 library needed.

It emits the same subset of the HDF5 format that those files use: a version-0 superblock,
version-1 object headers, groups as symbol tables (a version-1 B-tree over symbol table
nodes of at most eight entries, names in a local heap), contiguous datasets with version-1
dataspaces and version-3 layouts, IEEE little-endian floats, (real, imag) float compounds
for complex data, 32-bit integers, and scalar integer attributes.  Dataset dimensions are
written in HDF5 order, the reverse of the column-major Blitz extents (src/hdf5_interface.h
H5ArrayWrite: dimsf[i] = A.length(N - i - 1)).
"""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


def _float_type(size=4):
    if size == 4:
        return struct.pack("<B3sI", 0x11, bytes([0x20, 31, 0]), 4) + struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
    return struct.pack("<B3sI", 0x11, bytes([0x20, 63, 0]), 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)


def _int_type(size=4, signed=True):
    return struct.pack("<B3sI", 0x10, bytes([0x08 if signed else 0, 0, 0]), size) + struct.pack("<HH", 0, 8 * size)


def _complex_type(size=4):
    out = struct.pack("<B3sI", 0x16, bytes([2, 0, 0]), 2 * size)
    for k, name in enumerate((b"real", b"imag")):
        out += _pad8(name + b"\0") + struct.pack("<IB3sI4s16s", k * size, 0, b"", 0, b"", b"") + _float_type(size)
    return out


def _space(dims):
    return struct.pack("<BBBB4s", 1, len(dims), 0, 0, b"") + b"".join(struct.pack("<Q", int(d)) for d in dims)


def _msg(mtype, body):
    body = _pad8(body)
    return struct.pack("<HHB3s", mtype, len(body), 0, b"") + body


def _ohdr(msgs):
    blob = b"".join(msgs)
    return struct.pack("<BBHII", 1, 0, len(msgs), 1, len(blob)) + b"\0" * 4 + blob


class _File:
    def __init__(self):
        self.buf = bytearray(b"\0" * 96)  # superblock, filled last

    def alloc(self, data):
        at = len(self.buf)
        self.buf += _pad8(bytes(data))
        return at

    def reserve(self, n):
        at = len(self.buf)
        self.buf += b"\0" * (n + (-n % 8))
        return at


def _group(f, entries, attrs=None):
    """entries: name -> object header address; attrs: name -> int.  Returns (object header
    address, B-tree address, heap address)."""
    names = sorted(entries)
    heap = b"\0" * 8  # offset 0: the empty name
    offs = {}
    for n in names:
        offs[n] = len(heap)
        heap += _pad8(n.encode() + b"\0")
    heap_data = f.alloc(heap)
    heap_at = f.alloc(b"HEAP" + struct.pack("<B3sQQQ", 0, b"", len(heap), UNDEF, heap_data))
    snods = []
    for k in range(0, max(len(names), 1), 8):
        chunk = names[k:k + 8]
        body = b"SNOD" + struct.pack("<BBH", 1, 0, len(chunk))
        for n in chunk:
            body += struct.pack("<QQII16s", offs[n], entries[n], 0, 0, b"")
        snods.append((f.alloc(body), chunk))
    tree = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF)
    tree += struct.pack("<Q", 0)
    for at, chunk in snods:
        tree += struct.pack("<QQ", at, offs[chunk[-1]] if chunk else 0)
    tree_at = f.alloc(tree)
    msgs = [_msg(0x0011, struct.pack("<QQ", tree_at, heap_at))]
    for name, val in (attrs or {}).items():
        nm, tp, sp = name.encode() + b"\0", _int_type(), _space([])
        body = struct.pack("<BBHHH", 1, 0, len(nm), len(tp), len(sp)) + _pad8(nm) + _pad8(tp) + _pad8(sp)
        msgs.append(_msg(0x000C, body + struct.pack("<i", int(val))))
    return f.alloc(_ohdr(msgs)), tree_at, heap_at


def _dataset(f, arr, dims_hdf5):
    arr = np.ascontiguousarray(arr)
    if arr.dtype == np.complex64:
        tp = _complex_type(4)
    elif arr.dtype == np.complex128:
        tp = _complex_type(8)
    elif arr.dtype == np.float32:
        tp = _float_type(4)
    elif arr.dtype == np.float64:
        tp = _float_type(8)
    elif arr.dtype == np.int32:
        tp = _int_type(4)
    elif arr.dtype == np.uint64:
        tp = _int_type(8, signed=False)
    else:
        raise TypeError(arr.dtype)
    raw = arr.tobytes()
    data_at = f.alloc(raw)
    lay = struct.pack("<BBQQ", 3, 1, data_at, len(raw))
    return f.alloc(_ohdr([_msg(0x0001, _space(dims_hdf5)), _msg(0x0003, tp), _msg(0x0008, lay)]))


def write_mri_file(path, encodes, num_coils, traj_types=(1, 1, 1), dft_needed=(1, 1, 1)):
    """encodes: list of dicts with kx, ky, kz, kw (float32, shape (slices, projections,
    readout) in HDF5 order, i.e. the reference's (readout, projections, slices) arrays),
    optional kt, and kdata (num_coils, same shape) complex64."""
    f = _File()
    kd, gt = {}, {}
    for e, enc in enumerate(encodes):
        shape = enc["kx"].shape
        for key, name in (("kx", "KX_E%d"), ("ky", "KY_E%d"), ("kz", "KZ_E%d"), ("kw", "KW_E%d")):
            kd[name % e] = _dataset(f, enc[key].astype(np.float32), shape)
        kd["KT_E%d" % e] = _dataset(f, enc.get("kt", np.zeros(shape, np.float32)).astype(np.float32), shape)
        for c in range(num_coils):
            kd["KData_E%d_C%d" % (e, c)] = _dataset(f, enc["kdata"][c].astype(np.complex64), shape)
        gshape = shape[:-1]  # one value per readout
        for name in ("ECG_E%d", "RESP_E%d", "PREP_E%d", "TIME_E%d"):
            gt[name % e] = _dataset(f, np.zeros(gshape, np.float64), gshape)
        gt["CLOCK_E%d" % e] = _dataset(f, np.zeros(gshape, np.uint64), gshape)
    attrs = {"Num_Encodings": len(encodes), "Num_Coils": num_coils, "trajectory_typeX": traj_types[0],
             "trajectory_typeY": traj_types[1], "trajectory_typeZ": traj_types[2], "dft_neededX": dft_needed[0],
             "dft_neededY": dft_needed[1], "dft_neededZ": dft_needed[2]}
    kdata_at, _, _ = _group(f, kd, attrs)
    gating_at, _, _ = _group(f, gt)
    root_at, root_tree, root_heap = _group(f, {"Kdata": kdata_at, "Gating": gating_at})
    eof = len(f.buf)
    sb = b"\x89HDF\r\n\x1a\n" + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, 4, 16, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII", 0, root_at, 1, 0) + struct.pack("<QQ", root_tree, root_heap)
    assert len(sb) == 96
    f.buf[:96] = sb
    with open(path, "wb") as fh:
        fh.write(bytes(f.buf))
