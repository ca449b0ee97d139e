"""Minimal writer of the Pinco results archive (test infrastructure): one
chunk set, entries in the given order, continuations linked through the
register like the reference's ChunkRegister (ChunkRegister.cpp:152-233,
312-380; ChunkFileSet.cpp:58-224). Little-endian 8-byte size_t / long."""
import os
import struct

import numpy as np

from pinco_reader import MAGIC


def write_archive(data_dir, names, dims, formats, entries):
    """entries: list of (id, t_start, t_end, {name: array of shape (frames, sites)})."""
    os.makedirs(data_dir, exist_ok=True)
    hdr = bytearray(MAGIC) + bytes([1, len(names)])
    for n in names:
        hdr += bytes([len(n)]) + n.encode()
    for d in dims:
        hdr += struct.pack("<Q", len(d)) + struct.pack(f"<{len(d)}Q", *d)
    hdr += bytes(formats)
    first = len(hdr) + 16
    hdr += struct.pack("<qq", 16, first)
    files = [open(os.path.join(data_dir, f"variable{j}_1.cnk"), "wb") for j in range(len(names))]
    index = open(os.path.join(data_dir, "index_1.bin"), "wb")
    reg = bytearray(hdr)
    last_pos = {}
    for row, (tid, ts, te, data) in enumerate(entries):
        rec = [tid]
        for j, n in enumerate(names):
            arr = np.ascontiguousarray(data[n], dtype=np.float64 if formats[j] == 11 else np.complex128)
            off = files[j].tell()
            payload = arr.tobytes()
            files[j].write(struct.pack("<Q", len(payload)) + payload)
            rec += [arr.shape[0], off]
        index.write(struct.pack(f"<{len(rec)}Q", *rec))
        pos = len(reg)
        if tid in last_pos:  # link the previous entry of this trajectory to this one
            struct.pack_into("<Q", reg, last_pos[tid] + 24, pos)
        reg += struct.pack("<4Q", tid, 1, row, 0) + struct.pack("<2d", ts, te)
        last_pos[tid] = pos
    for f in files:
        f.close()
    index.close()
    with open(os.path.join(data_dir, "_register.bin"), "wb") as f:
        f.write(bytes(reg))
