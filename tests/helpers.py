"""Comparison helpers shared by the parity tests."""
import numpy as np


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def configs_for(w, **kw):
    """(oracle config, library config) for a workload dict."""
    from oracle import oracle as O
    from vpm_free_gb300 import VPMConfig
    args = dict(dpm=w["dpm"], box=w["box"])
    args.update(kw)
    return O.make_config(**args), VPMConfig.make(**args)


def fortran_records(path):
    """Payloads of a Fortran sequential unformatted file (4-byte length markers)."""
    import struct
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        rec = data[pos + 4:pos + 4 + n]
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        assert m == n, "broken record marker"
        out.append(rec)
        pos += 8 + n
    return out
