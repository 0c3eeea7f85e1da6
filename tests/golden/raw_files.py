"""Writers of nova's raw (comma-separated) POMDP / MDP file layout, used to
make loader fixtures from synthetic models (the layout read by
python/nova/file_loader.py:74-209)."""
import numpy as np


def _fmt(x):
    return repr(float(np.float32(x)))


def write_raw_pomdp(model, path, k=1, s0=0):
    """Rewards: k functions; function 0 is model['R'], the others are R + i."""
    n, ns, m, z, r, rz = (model[q] for q in ("n", "ns", "m", "z", "r", "rz"))
    lines = [",".join(str(v) for v in (n, ns, m, z, r, rz, k, s0, model["horizon"])) + "," + _fmt(model["gamma"])]
    for a in range(m):
        for s in range(n):
            lines.append(",".join(str(int(v)) for v in model["S"][s, a]))
    for a in range(m):
        for s in range(n):
            lines.append(",".join(_fmt(v) for v in model["T"][s, a]))
    for a in range(m):
        for o in range(z):
            lines.append(",".join(_fmt(v) for v in model["O"][a, :, o]))
    for i in range(k):
        for a in range(m):
            lines.append(",".join(_fmt(v + i) for v in model["R"][:, a]))
    for i in range(r):
        lines.append(",".join(str(int(v)) for v in model["Z"][i]))
    for i in range(r):
        lines.append(",".join(_fmt(v) for v in model["B"][i]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_raw_mdp(model, path, k=1, s0=0, goals=()):
    n, ns, m = model["n"], model["ns"], model["m"]
    lines = [",".join(str(v) for v in (n, ns, m, k, s0, len(goals), model["horizon"])) + "," + _fmt(model["gamma"])]
    lines.append(",".join(str(int(g)) for g in goals))
    for a in range(m):
        for s in range(n):
            lines.append(",".join(str(int(v)) for v in model["S"][s, a]))
    for a in range(m):
        for s in range(n):
            lines.append(",".join(_fmt(v) for v in model["T"][s, a]))
    for i in range(k):
        for a in range(m):
            lines.append(",".join(_fmt(v + i) for v in model["R"][:, a]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
