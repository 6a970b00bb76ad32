"""Reader and writer for the knng container file.

The reference engine reads ``/train`` from an HDF5 file and writes ``knns``,
``dists`` and five root attributes to ``results/<task>/apex_simd.h5``
(Aftab5550/SISAP-2026-task1 src/main.cpp:149-177, 459-480).  Without libhdf5
in the image, the same datasets and attributes are carried in a flat container
that the knng_main CLI and the oracle's H5Cpp shim both understand:

    magic  b"KNNGH5S1"
    record u32 tag (1 dataset, 2 string attribute, 3 float attribute)
           u32 name length, name bytes
           dataset: u32 type (1 f32, 2 i32, 3 f16, 4 i8), u32 rank, u64 dims[rank],
                    raw little-endian row-major data
           string : u64 length, bytes
           float  : f32
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"KNNGH5S1"
_TYPES = {1: np.float32, 2: np.int32, 3: np.float16, 4: np.int8}
_CODES = {np.dtype(v): k for k, v in _TYPES.items()}


def write(path, datasets=None, str_attrs=None, float_attrs=None):
    """Write datasets (name -> ndarray) and scalar attributes to ``path``."""
    with open(path, "wb") as f:
        f.write(MAGIC)
        for name, arr in (datasets or {}).items():
            arr = np.ascontiguousarray(arr)
            code = _CODES.get(arr.dtype)
            if code is None:
                raise TypeError(f"unsupported dtype {arr.dtype} for {name}")
            nb = name.lstrip("/").encode()
            f.write(struct.pack("<II", 1, len(nb)) + nb)
            f.write(struct.pack("<II", code, arr.ndim))
            f.write(struct.pack(f"<{arr.ndim}Q", *arr.shape))
            f.write(arr.astype(arr.dtype.newbyteorder("<"), copy=False).tobytes())
        for name, val in (str_attrs or {}).items():
            nb, vb = name.encode(), val.encode()
            f.write(struct.pack("<II", 2, len(nb)) + nb + struct.pack("<Q", len(vb)) + vb)
        for name, val in (float_attrs or {}).items():
            nb = name.encode()
            f.write(struct.pack("<II", 3, len(nb)) + nb + struct.pack("<f", float(val)))


def read(path, mmap=True):
    """Return (datasets, attrs) from a container or an HDF5 file (told apart by
    the signature; HDF5 goes through hdf5read).  Datasets are memory-mapped
    unless ``mmap`` is False."""
    datasets, attrs = {}, {}
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            import hdf5read

            ds, at = hdf5read.read(path)
            return ({k: np.array(v) for k, v in ds.items()} if not mmap else ds), at
        while True:
            hdr = f.read(8)
            if len(hdr) < 8:
                break
            tag, ln = struct.unpack("<II", hdr)
            name = f.read(ln).decode()
            if tag == 1:
                code, rank = struct.unpack("<II", f.read(8))
                shape = struct.unpack(f"<{rank}Q", f.read(8 * rank))
                dt = np.dtype(_TYPES[code])
                off = f.tell()
                count = int(np.prod(shape)) if rank else 1
                if mmap:
                    datasets[name] = np.memmap(path, dtype=dt, mode="r", offset=off, shape=shape)
                else:
                    datasets[name] = np.fromfile(f, dtype=dt, count=count).reshape(shape)
                f.seek(off + count * dt.itemsize)
            elif tag == 2:
                (n,) = struct.unpack("<Q", f.read(8))
                attrs[name] = f.read(n).decode()
            elif tag == 3:
                (attrs[name],) = struct.unpack("<f", f.read(4))
            else:
                raise ValueError(f"{path}: unknown record tag {tag}")
    return datasets, attrs
