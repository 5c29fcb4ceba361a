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
