"""Independent reader of the Pinco results archive (test infrastructure).

Byte layout of the reference's ChunkRegister / ChunkFileSet
(src/Base/FileFormats/PincoFormat/ChunkRegister.cpp:152-233, 312-380,
ChunkFileSet.cpp:58-224): little-endian 8-byte size_t / long.
"""
import os
import struct

import numpy as np

MAGIC = bytes([0x89, ord("P"), ord("N"), ord("C"), 0x0D, 0x0A, 0x1A, 0x0A])


def read_register(data_dir):
    b = open(os.path.join(data_dir, "_register.bin"), "rb").read()
    assert b[:8] == MAGIC, "bad magic"
    version = b[8]
    p = 9
    nd = b[p]
    p += 1
    names = []
    for _ in range(nd):
        ln = b[p]
        names.append(b[p + 1:p + 1 + ln].decode())
        p += 1 + ln
    dims = []
    for _ in range(nd):
        (D,) = struct.unpack_from("<Q", b, p)
        p += 8
        dims.append(list(struct.unpack_from(f"<{D}Q", b, p)))
        p += 8 * D
    formats = list(b[p:p + nd])
    p += nd
    extra_size, first = struct.unpack_from("<qq", b, p)
    p += 16
    assert first == p, (first, p)
    entries = []
    esz = 32 + extra_size
    while p + esz <= len(b):
        tid, cid, coff, cont = struct.unpack_from("<4Q", b, p)
        ts, te = struct.unpack_from("<2d", b, p + 32)
        entries.append({"id": tid, "chunk": cid, "row": coff, "cont": cont, "t_start": ts, "t_end": te, "pos": p})
        p += esz
    assert p == len(b), "trailing bytes in register"
    return {"version": version, "names": names, "dims": dims, "formats": formats, "entries": entries}


def read_entry(data_dir, reg, entry):
    nd = len(reg["names"])
    idx = open(os.path.join(data_dir, f"index_{entry['chunk']}.bin"), "rb").read()
    rowsz = 8 * (1 + 2 * nd)
    row = struct.unpack_from(f"<{1 + 2 * nd}Q", idx, entry["row"] * rowsz)
    assert row[0] == entry["id"]
    out = {}
    for j, name in enumerate(reg["names"]):
        nel, off = row[1 + 2 * j], row[2 + 2 * j]
        with open(os.path.join(data_dir, f"variable{j}_{entry['chunk']}.cnk"), "rb") as f:
            f.seek(off)
            (nbytes,) = struct.unpack("<Q", f.read(8))
            dtype = np.float64 if reg["formats"][j] == 11 else np.complex128
            data = np.frombuffer(f.read(nbytes), dtype=dtype)
        out[name] = (nel, data)
    return out


def read_trajectory(data_dir, traj_id):
    """All entries of one trajectory in register order: (traj frames
    concatenated, the other datasets of the last entry, entries); the frame
    series work / area (float64) are concatenated into the second result."""
    reg = read_register(data_dir)
    ents = [e for e in reg["entries"] if e["id"] == traj_id]
    frames, real, series = [], {}, {}
    for e in ents:
        d = read_entry(data_dir, reg, e)
        for name, (nel, data) in d.items():
            if name == "traj":
                frames.append(data.reshape(nel, -1))
            elif name in ("work", "area"):
                series.setdefault(name, []).append(data.reshape(nel, -1))
            else:
                real[name] = data
    for name, parts in series.items():
        real[name] = np.concatenate(parts)
    return (np.concatenate(frames) if frames else None), real, ents


def read_times(path):
    lines = open(path).read().strip().split("\n")
    assert lines[0].startswith("%\tformat:real")
    return np.array([float(x) for x in lines[1:]])
