"""Loaders for the committed golden fixtures (tests/golden)."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def small_cases():
    out = {}
    for path in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        name = os.path.basename(path)[:-4]
        if name == "ref_sample_16x16" or name.startswith(("vpred", "proxy", "signs", "cw", "mct", "nlt")):
            continue
        z = np.load(path)
        w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc = [int(x) for x in z["params"]]
        out[name] = dict(w=w, h=h, d=d, fmt=fmt, bpp_num=bn, bpp_den=bd, v=v, hh=hh, q=q, sl=sl, sig=sig, rc=rc,
                         planes=[z["in%d" % i] for i in range(4) if "in%d" % i in z],
                         bs=z["bs"], dec=[z["dec%d" % i] for i in range(4) if "dec%d" % i in z])
    return out


def proxy_cases():
    """Codestreams of the small cases with the reference decoder's half (1)
    or quarter (2) resolution output."""
    out = {}
    for path in sorted(glob.glob(os.path.join(GOLDEN, "proxy*.npz"))):
        z = np.load(path)
        out[os.path.basename(path)[:-4]] = dict(proxy=int(z["proxy"][0]), bs=z["bs"],
                                                dec=[z["dec%d" % i] for i in range(4) if "dec%d" % i in z])
    return out


def sign_cases():
    """Codestreams of the reference encoder with separate sign sub-packets,
    with their inputs and the reference decoder's planes."""
    out = {}
    for path in sorted(glob.glob(os.path.join(GOLDEN, "signs*.npz"))):
        z = np.load(path)
        out[os.path.basename(path)[:-4]] = dict(params=[int(x) for x in z["params"]], bs=z["bs"],
                                                planes=[z["in%d" % i] for i in range(4) if "in%d" % i in z],
                                                dec=[z["dec%d" % i] for i in range(4) if "dec%d" % i in z])
    return out


def cw_cases():
    """Multi-column precinct codestreams (Cw > 0) made by the oracle's
    encoder, with the reference decoder's planes."""
    out = {}
    for path in sorted(glob.glob(os.path.join(GOLDEN, "cw*.npz"))):
        z = np.load(path)
        out[os.path.basename(path)[:-4]] = dict(params=[int(x) for x in z["params"]], bs=z["bs"],
                                                dec=[z["dec%d" % i] for i in range(4) if "dec%d" % i in z])
    return out


def mct_cases():
    """Colour transform (Cpih = 1) and output non-linearity codestreams made
    by the oracle's encoder, with the reference decoder's planes at full
    and half resolution."""
    out = {}
    for path in sorted(glob.glob(os.path.join(GOLDEN, "mct*.npz")) + glob.glob(os.path.join(GOLDEN, "nlt*.npz"))):
        z = np.load(path)
        out[os.path.basename(path)[:-4]] = dict(params=[int(x) for x in z["params"]], bs=z["bs"],
                                                dec=[z["dec%d" % i] for i in range(4) if "dec%d" % i in z],
                                                proxy=[z["proxy%d" % i] for i in range(4) if "proxy%d" % i in z])
    return out


def vpred_cases():
    """Codestreams of the reference encoder with vertical prediction, with
    their inputs and the reference decoder's planes."""
    out = {}
    for path in sorted(glob.glob(os.path.join(GOLDEN, "vpred*.npz"))):
        z = np.load(path)
        out[os.path.basename(path)[:-4]] = dict(params=[int(x) for x in z["params"]], bs=z["bs"],
                                                planes=[z["in%d" % i] for i in range(4) if "in%d" % i in z],
                                                dec=[z["dec%d" % i] for i in range(4) if "dec%d" % i in z])
    return out


def ref_sample():
    z = np.load(os.path.join(GOLDEN, "ref_sample_16x16.npz"))
    return z["bs"], int(z["frame_size"][0]), [z["dec%d" % i] for i in range(4) if "dec%d" % i in z]


def full_size():
    with open(os.path.join(GOLDEN, "full_size.json")) as fh:
        return json.load(fh)


def full_planes(case):
    import jxs_synth as S

    if case["kind"] == "4k":
        return S.frame_4k_10bit(case["seed"], case["frame"])
    if case["kind"] == "8k":
        return S.frame_8k_14bit(case["seed"])
    return S.frame(case["w"], case["h"], case["d"], case["fmt"], seed=case["seed"])
