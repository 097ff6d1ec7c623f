"""Reader for the flat record files written by oracle/ref_driver.cpp (test infrastructure)."""
import numpy as np

_DT = {"f8": np.float64, "u4": np.uint32}


def read_refbin(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        end = data.index(b"\n", pos)
        name, dt, cnt = data[pos:end].decode().split()
        pos = end + 1
        dtype = np.dtype(_DT[dt])
        n = int(cnt)
        out[name] = np.frombuffer(data, dtype=dtype, count=n, offset=pos).copy()
        pos += n * dtype.itemsize
    return out
