"""Oracle restatement of the basis handling of hqc.

Follows ``hqc/basis/parse.py:116-239`` (CP2K-format parser and radial
normalisation) and ``hqc/pbc/solver.py:109-151`` / ``hqc/pbc/gto.py:72-300``
(cartesian-to-spherical scaling: s * 1/sqrt(4 pi), p * sqrt(3/(4 pi))).
Test infrastructure only.
"""
import json
import os

import numpy as np

_TABLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "hqc_gb300", "basis", "gth_h.json")


def basis_block(name):
    """CP2K text block for hydrogen in basis ``name`` (e.g. 'gth-dzv')."""
    with open(_TABLE) as fh:
        table = json.load(fh)
    if name not in table:
        raise FileNotFoundError(f"no hydrogen entry for basis '{name}'")
    return table[name]


def _double_factorial(n):
    return 1 if n <= 0 else n * _double_factorial(n - 2)


def parse_block(text):
    """Return list of (quant_num, coeff) per set, like parse_quant_num/parse_gto."""
    lines = [ln.strip() for ln in text.split("\n") if ln.strip()]
    # lines[0] '#BASIS SET', lines[1] 'H NAME', lines[2] num_sets
    nsets = int(lines[2])
    out = []
    pos = 3
    for _ in range(nsets):
        q = np.array([int(w) for w in lines[pos].split()])
        nprim = q[3]
        coeff = np.array([[float(w) for w in lines[pos + 1 + k].split()] for k in range(nprim)])
        out.append((q, coeff))
        pos += nprim + 1
    return out


def normalize(sets):
    """Radial normalisation of every contraction column (parse.py:192-239)."""
    res = []
    for q, c in sets:
        alpha = c[:, 0]
        asum = alpha[:, None] + alpha[None, :]
        aprod = alpha[:, None] * alpha[None, :]
        cols = [alpha]
        col = 1
        lmin, lmax = q[1], q[2]
        for l in range(lmin, lmax + 1):
            const = 2.0 ** (l + 1.75) / np.pi ** 0.25 / np.sqrt(_double_factorial(2 * l + 1))
            for _ in range(q[4 + l - lmin]):
                ci = c[:, col]
                norm = (2.0 ** (l + 1.5) * np.einsum("i,j,ij,ij", ci, ci, asum ** (-l - 1.5),
                                                      aprod ** (l / 2 + 0.75))) ** -0.5
                cols.append(ci * alpha ** (l / 2 + 0.75) * const * norm)
                col += 1
        res.append((q, np.stack(cols, axis=1)))
    return res


class Basis:
    """Per-atom AO table.

    alpha: (n_prim,) all primitive exponents, sets concatenated.
    coef:  (n_ao_atom, n_prim) contraction coefficient of each AO including the
           cartesian-to-spherical factor (zero for primitives of other sets).
    l, cart: (n_ao_atom,) angular momentum and cartesian direction (p only).
    AO order per atom: every s contraction, then every p contraction as x,y,z
    (the order of ``hqc/pbc/solver.py:307-321``; for the supported hydrogen
    bases it equals the grid order of ``hqc/pbc/gto.py:268-288``).
    """

    def __init__(self, name):
        sets = normalize(parse_block(basis_block(name)))
        lmin = min(q[1] for q, _ in sets)
        lmax = max(q[2] for q, _ in sets)
        if lmin != 0:
            raise ValueError("l_min != 0")
        if lmax > 1:
            raise ValueError("l_max > 1 is not supported yet.")
        self.alpha = np.concatenate([c[:, 0] for _, c in sets])
        nprim = len(self.alpha)
        rows, ls, carts = [], [], []
        off = 0
        seen_p = False
        for q, c in sets:
            col = 1
            for l in range(q[1], q[2] + 1):
                for _ in range(q[4 + l - q[1]]):
                    full = np.zeros(nprim)
                    full[off:off + c.shape[0]] = c[:, col]
                    col += 1
                    if l == 0:
                        if seen_p:
                            raise ValueError("s contraction after a p contraction is not supported")
                        rows.append(full / np.sqrt(4 * np.pi))
                        ls.append(0)
                        carts.append(0)
                    else:
                        seen_p = True
                        for d in range(3):
                            rows.append(full * np.sqrt(3 / (4 * np.pi)))
                            ls.append(1)
                            carts.append(d)
            off += c.shape[0]
        self.coef = np.array(rows)
        self.l = np.array(ls)
        self.cart = np.array(carts)
        self.lmax = lmax
        self.nao = len(rows)
