"""Writers of small synthetic Cassandra-format POMDP files for the loader
fixtures. Each file exercises a set of the format's statements as the
reference's loader reads them (python/nova/file_loader.py:211-588): names or
counts, start distributions / single state / include / exclude, T and O as
matrices, rows and entries with '*' wildcards, "uniform" and "identity",
redefinitions, and R statements whose values are averaged (one number, a
row, a matrix)."""
import numpy as np


def _num(rng, lo=0.0, hi=1.0):
    return "%.7g" % rng.uniform(lo, hi)


def _dist(rng, k, zero_at=()):
    w = rng.exponential(size=k)
    for j in (zero_at if isinstance(zero_at, tuple) else (zero_at,)):
        w[j] = 0.0
    w = w / w.sum()
    return ["%.9g" % x for x in w]


def write_named(path, seed=1):
    """Named states, actions and observations; matrix, identity and uniform
    transitions; per-successor observation rows; wildcard rewards with
    redefinitions; comments; a few CRLF line endings."""
    rng = np.random.default_rng(seed)
    S = ["left", "mid", "right", "far"]
    A = ["stay", "go", "reset"]
    Z = ["ping", "pong", "none"]
    L = ["# synthetic model with named symbols", "", "discount: 0.93", "values: reward",
         "states: " + " ".join(S), "actions: " + " ".join(A), "observations: " + " ".join(Z), "",
         "start:", " ".join(_dist(rng, 4)), "", "T: stay", "identity", "", "T: reset", "uniform", "", "T: go"]
    for s in range(4):
        L.append(" ".join(_dist(rng, 4, zero_at=((s + 1) % 4, (s + 2) % 4))))
    # A row statement appends to the matrix's entries of (far, go).
    L += ["", "T: go : far", " ".join(_dist(rng, 4, zero_at=(1, 2)))]
    L += ["", "O: stay", "uniform", "", "O: go"]
    for s in range(4):
        L.append(" ".join(_dist(rng, 3)))
    for s in S:
        L += ["O: reset : %s" % s, " ".join(_dist(rng, 3))]
    L += ["O: reset : mid : pong %s" % _num(rng)]
    L += ["", "R: * : * : * : * %s  # everything" % _num(rng, -1, 0)]
    for a in A:
        for s in S[:3]:
            L.append("R: %s : %s : * : * %s" % (a, s, _num(rng, -5, 5)))
    L.append("R: go : mid : * : * %s" % _num(rng, -5, 5))  # redefined
    text = "\n".join(L[:10]) + "\r\n" + "\r\n".join(L[10:14]) + "\n" + "\n".join(L[14:]) + "\n"
    with open(path, "w", newline="") as f:
        f.write(text)


def write_counts(path, seed=2):
    """Counted symbols; start include; entry and row transitions with
    wildcards (duplicates append); entry observations; a reward matrix whose
    mean goes through numpy's pairwise summation."""
    rng = np.random.default_rng(seed)
    n, m, z = 6, 3, 2
    L = ["discount: 0.9", "states: %d" % n, "actions: %d" % m, "observations: %d" % z,
         "start include: 1 3 4"]
    for a in range(m):
        for s in range(n):
            row = _dist(rng, n, zero_at=((a + s) % n, (a + s + 3) % n))
            L += ["T: %d : %d" % (a, s), " ".join(row)]
    L.append("T: * : 2 : 0 %s" % _num(rng, 0.01, 0.2))
    L.append("T: 1 : * : 4 %s" % _num(rng, 0.01, 0.2))
    L.append("T: 1 : 3 : 3 0")  # zero probability: nothing appended
    for a in range(m):
        for s in range(n):
            p = rng.uniform(0.05, 0.95)
            L.append("O : %d : %d : 0 %.8g" % (a, s, p))
            L.append("O : %d : %d : 1 %.8g" % (a, s, 1.0 - p))
    L.append("O : * : 4 : * 0.5")
    L.append("R: * : * : * : * -1")
    L.append("R: 2 : 3")
    for _ in range(4):
        L.append(" ".join(_num(rng, -10, 10) for _ in range(5)))
    L.append("R: 0 : * : * %s" % _num(rng, -3, 3))
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def write_exclude(path, seed=3):
    """start exclude; a transition matrix for every action through '*';
    reward rows of 11 and 17 values."""
    rng = np.random.default_rng(seed)
    S = ["s%d" % i for i in range(6)]
    L = ["discount: 0.97", "states: " + " ".join(S), "actions: north south", "observations: 3",
         "start exclude: s0 s4", "T: *"]
    for s in range(6):
        L.append(" ".join(_dist(rng, 6, zero_at=s)))
    L += ["O: *", "uniform", "O: south : s5", "0.2 0.3 0.5"]
    L += ["R: north : s1 : *", " ".join(_num(rng, -2, 2) for _ in range(11))]
    L += ["R: south : * : s2", " ".join(_num(rng, -2, 2) for _ in range(17))]
    L += ["R: north : s5 : * : * 4.25"]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def write_single_start(path, seed=4):
    """A single start state by name, no discount statement (0.9)."""
    rng = np.random.default_rng(seed)
    L = ["states: a b c", "actions: x y", "observations: o1 o2", "start: b", "T: x", "identity", "T: y", "uniform",
         "O: *", "uniform", "R: x : * : * : * %s" % _num(rng, -1, 1), "R: y : c : * : * %s" % _num(rng, 1, 2)]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def write_long_rows(path):
    """Entry statements that append a successor list longer than n: the
    reference's pomdp_initialize_cpu rejects ns > n and loading fails."""
    L = ["states: 2", "actions: 1", "observations: 1", "start: 0.5 0.5", "T: 0", "identity", "T: 0 : 0 : 0 0.5",
         "T: 0 : 0 : 1 0.5", "O: 0", "uniform", "R: 0 : * : * : * 1", "R: 0 : 1 : * : * 2"]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def write_start_uniform(path):
    """'start: uniform': the reference's test of the start statement never
    matches, 'uniform' is looked up as a state name, and loading fails."""
    L = ["states: 2", "actions: 1", "observations: 1", "start: uniform", "T: 0", "identity", "O: 0", "uniform",
         "R: 0 : * : * : * 1", "R: 0 : 1 : * : * 2"]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def write_no_reward(path):
    """No R statement: the reference never sets its horizon and fails."""
    L = ["states: 2", "actions: 1", "observations: 1", "start: 0.5 0.5", "T: 0", "identity", "O: 0", "uniform"]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


WRITERS = {"cass_named": write_named, "cass_counts": write_counts, "cass_exclude": write_exclude,
           "cass_single_start": write_single_start, "cass_start_uniform": write_start_uniform,
           "cass_no_reward": write_no_reward, "cass_long_rows": write_long_rows}
