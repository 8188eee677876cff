"""Loaders for the committed golden fixtures (see golden/make_golden.py)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def parse_cli_args(args):
    """Map a flct argv tail (deltat deltas sigma [options]) to keyword
    parameters, following the reference's option grammar (flct.c:370-487)."""
    kw = dict(deltat=float(args[0]), deltas=float(args[1]), sigma=float(args[2]))
    rest = [str(a) for a in args[3:]]
    i = 0
    while i < len(rest):
        a = rest[i]
        if a.startswith("-h"):
            kw["hires"] = True
        elif a.startswith("-t") and i + 1 < len(rest):
            s = rest[i + 1]
            kw["thresh_abs"] = "a" in s
            kw["thresh"] = float(s.split("a")[0])
        elif a.startswith("-k") and i + 1 < len(rest):
            kw["kr"] = float(rest[i + 1])
        elif a.startswith("-s") and i + 1 < len(rest):
            s = rest[i + 1]
            kw["interpolate"] = "i" in s
            s = s.split("i")[0]
            q = p = 0
            if "q" in s:
                s, qs = s.split("q", 1)
                q = int(qs)
            if "p" in s:
                s, ps = s.split("p", 1)
                p = int(ps)
            kw["skip"], kw["poffset"], kw["qoffset"] = int(s), p, q
            if kw["skip"] == 0:
                kw["skip"] = -1  # "-s 0" is the reference's non-positive-skip error
        i += 1
    return kw


def cli_cases():
    z = load("ref_cli_cases.npz")
    out = []
    for idx, (name, args, rc) in enumerate(json.loads(str(z["index"]))):
        f1 = z[f"c{idx}_f1"].astype(np.float64)
        f2 = z[f"c{idx}_f2"].astype(np.float64)
        ref = None
        if rc == 0:
            ref = tuple(z[f"c{idx}_{n}"].astype(np.float64) for n in ("vx", "vy", "vm"))
        out.append((name, args, rc, f1, f2, ref))
    return out


def window_cases():
    z = load("ref_window_cases.npz")
    out = []
    for g in range(int(z["count"])):
        meta = json.loads(str(z[f"w{g}_meta"]))
        out.append((meta["n"], meta["kr"], z[f"w{g}_g1"].astype(np.float64),
                    z[f"w{g}_g2"].astype(np.float64), z[f"w{g}_sx"], z[f"w{g}_sy"]))
    return out
