"""Gauss-Legendre nodal basis tables for the DG operators (row sizes 2-8).

The tables are the constant operators the reference's kernels consume through
``hexed::Basis`` (include/Basis.hpp:14-63, src/Basis.cpp:6-14) and that the
reference generates at build time (script/Basis.py:10-204, script/auto_generate.py:61-160):

* ``node``/``weight``  Gauss-Legendre rule mapped to [0, 1], weights summing to 1
* ``diff_mat``         D[i][j] = derivative of Lagrange polynomial j at node i
* ``boundary``         B[s][j] = Lagrange polynomial j evaluated at s in {0, 1}
* ``orthogonal``       Legendre polynomials at the nodes, unit norm under the rule
* ``filter``           modal low-pass: sum_k phi_k(x_i) 0.5^k phi_k(x_j) w_j
* ``prolong``          P_h[i][j] = L_j((x_i + h)/2), h in {0, 1}
* ``restrict``         R_h[i][j] = w_j/2 L_i((x_j + h)/2) / w_i (L2 projection)
* ``eigenvals``        minimum real part of the eigenvalues of the 1-D periodic
                       advection and diffusion DG operators on 16 unit elements
                       (script/Basis.py:158-204); they set ``max_cfl`` and the
                       diffusive time-step limit.

All matrices are returned row-major as ``M[i][j]`` (first index = result node).
The arithmetic runs in 50-digit mpmath and is rounded to the nearest double once.
The eigenvalue step is the only float64 computation, as in the reference.

Running this module as a script regenerates ``csrc/basis_tables.h`` and
``basis_tables.json`` next to it. mpmath is needed only for regeneration; the
library and the tests read the committed outputs.
"""
from __future__ import annotations

import json
import os

import numpy as np

MIN_ROW_SIZE = 2
MAX_ROW_SIZE = 8
QUADRATIC_SAFETY = 0.9  # Gauss_legendre::quadratic_safety (include/Gauss_legendre.hpp:18)
N_EIG_ELEM = 16

_HERE = os.path.dirname(os.path.abspath(__file__))
JSON_PATH = os.path.join(_HERE, "basis_tables.json")
HEADER_PATH = os.path.join(_HERE, "csrc", "basis_tables.h")


def _gauss_legendre_rule(n, mp):
    """Nodes ascending in [0, 1] and weights summing to 1, by Newton on P_n."""
    nodes, weights = [], []
    for k in range(n):
        # Chebyshev-like initial guess for the k-th root of P_n on [-1, 1] (descending)
        x = mp.cos(mp.pi * (k + mp.mpf(3) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p0, p1 = mp.mpf(1), x
            for m in range(2, n + 1):
                p0, p1 = p1, ((2 * m - 1) * x * p1 - (m - 1) * p0) / m
            pn = p1 if n >= 1 else p0
            pnm1 = p0
            dp = n * (x * pn - pnm1) / (x * x - 1)
            dx = pn / dp
            x -= dx
            if abs(dx) < mp.mpf(10) ** (-(mp.mp.dps - 5)):
                break
        p0, p1 = mp.mpf(1), x
        for m in range(2, n + 1):
            p0, p1 = p1, ((2 * m - 1) * x * p1 - (m - 1) * p0) / m
        dp = n * (x * p1 - p0) / (x * x - 1)
        w = 2 / ((1 - x * x) * dp * dp)
        nodes.append((x + 1) / 2)
        weights.append(w / 2)
    order = sorted(range(n), key=lambda i: nodes[i])
    return [nodes[i] for i in order], [weights[i] for i in order]


def _lagrange(nodes, j, x):
    r = 1
    for m, xm in enumerate(nodes):
        if m != j:
            r *= (x - xm) / (nodes[j] - xm)
    return r


def _lagrange_deriv(nodes, i, j):
    """d L_j / dx at node i."""
    n = len(nodes)
    if i == j:
        s = 0
        for m in range(n):
            if m != i:
                s += 1 / (nodes[i] - nodes[m])
        return s
    num = 1
    for m in range(n):
        if m != j:
            num /= (nodes[j] - nodes[m])
            if m != i:
                num *= (nodes[i] - nodes[m])
    return num


def _legendre_at(deg, t):
    p0, p1 = 1, t
    if deg == 0:
        return p0
    for m in range(2, deg + 1):
        p0, p1 = p1, ((2 * m - 1) * t * p1 - (m - 1) * p0) / m
    return p1


def _eigenvals(diff, bound_lo, bound_hi, weights, n_elem=N_EIG_ELEM):
    """Minimum real parts of the periodic 1-D DG advection and diffusion operators.

    Restates script/Basis.py:158-204 (the ``discon`` matrix there is unused).
    ``bound_lo[j]`` = L_j(0) and ``bound_hi[j]`` = L_j(1).
    """
    rs = len(weights)
    n = n_elem * rs
    local_grad = np.zeros((n, n))
    avrg = np.zeros((n, n))
    jump = np.zeros((n, n))
    at = [bound_lo, bound_hi]  # at[s][j] = L_j(s)
    for e in range(n_elem):
        for i in range(rs):
            for j in range(rs):
                local_grad[e * rs + i, e * rs + j] = diff[i][j]
                for si in (0, 1):
                    for sj in (0, 1):
                        row = ((e + si) % n_elem) * rs + i
                        col = ((e + sj) % n_elem) * rs + j
                        b = at[1 - sj][j] * at[1 - si][i] / weights[i]
                        avrg[row, col] += 0.5 * (2 * sj - 1) * b
                        jump[row, col] += 0.5 * (1 - 2 * (sj == si)) * b
    advection = -local_grad - avrg + jump
    grad = local_grad + avrg
    diffusion = grad @ grad
    return [float(np.linalg.eigvals(m).real.min()) for m in (advection, diffusion)]


def compute_tables(row_size, dps=50):
    import mpmath as mp

    mp.mp.dps = dps
    nodes, weights = _gauss_legendre_rule(row_size, mp)
    rs = row_size
    diff = [[_lagrange_deriv(nodes, i, j) for j in range(rs)] for i in range(rs)]
    bound = [[_lagrange(nodes, j, mp.mpf(s)) for j in range(rs)] for s in (0, 1)]
    ortho = []
    for deg in range(rs):
        vals = [_legendre_at(deg, 2 * x - 1) for x in nodes]
        norm = mp.sqrt(sum(v * v * w for v, w in zip(vals, weights)))
        ortho.append([v / norm for v in vals])
    filt = [[sum(ortho[k][i] * mp.mpf("0.5") ** k * ortho[k][j] * weights[j] for k in range(rs))
             for j in range(rs)] for i in range(rs)]
    prolong = [[[_lagrange(nodes, j, (nodes[i] + h) / 2) for j in range(rs)] for i in range(rs)]
               for h in (0, 1)]
    restrict = [[[weights[j] / 2 * _lagrange(nodes, i, (nodes[j] + h) / 2) / weights[i]
                  for j in range(rs)] for i in range(rs)] for h in (0, 1)]

    def f(x):
        return float(x)

    def fl(v):
        if isinstance(v, list):
            return [fl(x) for x in v]
        return f(v)

    t = {
        "row_size": rs,
        "node": fl(nodes),
        "weight": fl(weights),
        "diff_mat": fl(diff),
        "boundary": fl(bound),
        "orthogonal": fl(ortho),
        "filter": fl(filt),
        "prolong": fl(prolong),
        "restrict": fl(restrict),
    }
    # The reference feeds 20-significant-digit decimal values into the float64
    # eigenvalue problem; the nearest doubles used here differ by < 1 ulp.
    eig = _eigenvals(t["diff_mat"], t["boundary"][0], t["boundary"][1], t["weight"])
    t["eigenvals"] = eig
    t["max_cfl"] = -2 * QUADRATIC_SAFETY / eig[0]
    t["step_ratio"] = 0.5 / QUADRATIC_SAFETY
    t["min_eig_diffusion"] = eig[1]
    return t


def generate(path_json=JSON_PATH, path_header=HEADER_PATH):
    tables = {str(rs): compute_tables(rs) for rs in range(MIN_ROW_SIZE, MAX_ROW_SIZE + 1)}
    with open(path_json, "w") as fh:
        json.dump(tables, fh, indent=1)
    _write_header(tables, path_header)
    return tables


def _c(v):
    return repr(float(v))


def _write_header(tables, path):
    lines = [
        "// Generated by hexed_gb300/basis.py: Gauss-Legendre DG basis tables, row sizes "
        f"{MIN_ROW_SIZE}-{MAX_ROW_SIZE}.",
        "// All matrices row-major, first index = result node. Do not edit by hand.",
        "#pragma once",
        f"#define HEXED_MIN_ROW_SIZE {MIN_ROW_SIZE}",
        f"#define HEXED_MAX_ROW_SIZE {MAX_ROW_SIZE}",
        "namespace hexed_tables {",
    ]
    for rs_s, t in tables.items():
        rs = int(rs_s)

        def arr(name, vals):
            flat = np.asarray(vals, dtype=np.float64).ravel()
            body = ", ".join(_c(x) for x in flat)
            lines.append(f"static const double {name}{rs}[{flat.size}] = {{{body}}};")

        arr("node", t["node"])
        arr("weight", t["weight"])
        arr("diff_mat", t["diff_mat"])
        arr("boundary", t["boundary"])
        arr("orthogonal", t["orthogonal"])
        arr("filter", t["filter"])
        arr("prolong", t["prolong"])
        arr("restrict_", t["restrict"])
        lines.append(f"static const double max_cfl{rs} = {_c(t['max_cfl'])};")
        lines.append(f"static const double min_eig_diffusion{rs} = {_c(t['min_eig_diffusion'])};")
    lines.append(f"static const double step_ratio = {_c(0.5 / QUADRATIC_SAFETY)};")
    lines.append("}  // namespace hexed_tables")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


_CACHE = None


def load_tables():
    """Committed tables, keyed by row size (int)."""
    global _CACHE
    if _CACHE is None:
        with open(JSON_PATH) as fh:
            raw = json.load(fh)
        _CACHE = {int(k): v for k, v in raw.items()}
    return _CACHE


class Basis:
    """numpy view of one row size's tables (mirrors hexed::Basis accessors)."""

    def __init__(self, row_size):
        t = load_tables()[row_size]
        self.row_size = row_size
        self._t = t
        self.nodes = np.array(t["node"])
        self.node_weights = np.array(t["weight"])
        self.diff_mat = np.array(t["diff_mat"])
        self.boundary = np.array(t["boundary"])
        self.filter = np.array(t["filter"])
        self.prolong = [np.array(t["prolong"][h]) for h in (0, 1)]
        self.restrict = [np.array(t["restrict"][h]) for h in (0, 1)]
        self.max_cfl = t["max_cfl"]
        self.step_ratio = t["step_ratio"]
        self.min_eig_diffusion = t["min_eig_diffusion"]

    def orthogonal(self, degree):
        return np.array(self._t["orthogonal"][degree])

    def interpolate(self, sample):
        """interp[i][j] = L_j(sample[i])  (src/Basis.cpp:20-31)."""
        sample = np.asarray(sample, dtype=np.float64)
        out = np.ones((sample.size, self.row_size))
        for i in range(self.row_size):
            for j in range(self.row_size):
                if i != j:
                    out[:, i] *= (sample - self.nodes[j]) / (self.nodes[i] - self.nodes[j])
        return out


if __name__ == "__main__":
    generate()
    print("wrote", JSON_PATH, HEADER_PATH)
