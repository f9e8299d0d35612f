"""TEST INFRASTRUCTURE: reader for the "MTB1" named-array files written by the oracle harness."""
import struct

import numpy as np

_DT = {ord("d"): np.float64, ord("f"): np.float32, ord("i"): np.int32, ord("q"): np.int64}


def read_mtb(path: str) -> dict:
    out = {}
    with open(path, "rb") as fh:
        if fh.read(4) != b"MTB1":
            raise ValueError("not an MTB1 file")
        while True:
            hdr = fh.read(4)
            if not hdr:
                break
            (n,) = struct.unpack("<I", hdr)
            name = fh.read(n).decode()
            dt = _DT[fh.read(1)[0]]
            (nd,) = struct.unpack("<I", fh.read(4))
            dims = struct.unpack("<" + "Q" * nd, fh.read(8 * nd))
            cnt = int(np.prod(dims)) if nd else 1
            data = np.frombuffer(fh.read(cnt * np.dtype(dt).itemsize), dtype=dt).reshape(dims)
            out[name] = data.copy()
    return out
