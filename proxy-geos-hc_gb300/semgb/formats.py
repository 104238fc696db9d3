"""Pure-numpy readers of the SEMTRC01 (traces) and SEMSNP01 (snapshot) containers written by
sem_traces_write / sem_solver_write_snapshot: 8-byte magic, little-endian uint64 header length,
UTF-8 JSON header, zero padding to 64 bytes, little-endian float32 samples."""
from __future__ import annotations

import json

import numpy as np


def _read(path, magic: bytes):
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:8] != magic:
        raise ValueError(f"{path}: not a {magic.decode()} file")
    n = int.from_bytes(raw[8:16], "little")
    header = json.loads(raw[16:16 + n].decode("utf-8"))
    off = (16 + n + 63) // 64 * 64
    return header, np.frombuffer(raw, dtype="<f4", offset=off)


def read_traces(path):
    """(header dict, traces [n_samples][n_traces]) -- the file is trace-major."""
    h, data = _read(path, b"SEMTRC01")
    ns, nt = h["n_samples"], h["n_traces"]
    return h, data[:ns * nt].reshape(nt, ns).T.astype(np.float32)


def read_snapshot(path):
    """(header dict, plane [nz][nx])."""
    h, data = _read(path, b"SEMSNP01")
    return h, data[:h["nx"] * h["nz"]].reshape(h["nz"], h["nx"]).astype(np.float32)
