"""Reader for the binary records written by oracle/ref/harness.c.

Record: char name[32]; char dtype[4] ("f8", "i4", "u1"); int64 n; n values.
"""
import numpy as np

_DT = {b"f8": np.float64, b"i4": np.int32, b"u1": np.uint8}


def read_dump(path):
    out = {}
    with open(path, "rb") as fh:
        buf = fh.read()
    pos = 0
    while pos < len(buf):
        name = buf[pos:pos + 32].split(b"\0", 1)[0].decode()
        dt = buf[pos + 32:pos + 36].split(b"\0", 1)[0]
        n = int(np.frombuffer(buf, np.int64, 1, pos + 36)[0])
        pos += 44
        dtype = np.dtype(_DT[dt])
        out[name] = np.frombuffer(buf, dtype, n, pos).copy()
        pos += n * dtype.itemsize
    return out
