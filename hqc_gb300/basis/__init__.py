"""Hydrogen GTH basis sets: CP2K-format parsing and normalisation.

Mirrors the reference's ``hqc/basis/parse.py`` API (``load_as_str``,
``parse_quant_num``, ``parse_gto``, ``normalize_gto_coeff``; lines 32-239) on
the table ``gth_h.json`` (the hydrogen blocks of the reference's basis files,
see ``make_basis_table.py``), and adds ``basis_tables``: the per-atom AO table
the engine consumes (contraction coefficients with the cartesian-to-spherical
factors of ``hqc/pbc/solver.py:109-151``).
"""
import json
import os

import numpy as np

_TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gth_h.json")
_TABLE = None


def _table():
    global _TABLE
    if _TABLE is None:
        with open(_TABLE_PATH) as fh:
            _TABLE = json.load(fh)
    return _TABLE


def available():
    return sorted(_table())


def load_as_str(element, basis):
    """Basis block of ``element`` as a CP2K-format string (parse.py:32-64)."""
    if element != "H":
        raise ValueError(f"No '{element}' in '{basis}': only hydrogen is tabulated.")
    table = _table()
    if basis not in table:
        raise FileNotFoundError(f"No '{basis}.dat' basis file for hydrogen.")
    return table[basis]


def _lines(text):
    return [ln.strip() for ln in text.split("\n") if ln.strip()]


def parse_quant_num(element, basis):
    """Per set: [n, l_min, l_max, n_prim, n_contr(l_min), ...] (parse.py:116-140)."""
    ls = _lines(load_as_str(element, basis))
    nsets = int(ls[2])
    out, pos = [], 3
    for _ in range(nsets):
        q = np.array([int(v) for v in ls[pos].split()])
        if len(q) != 5 + q[2] - q[1]:
            raise ValueError(f"Line {ls[pos]} has incorrect number of l orbitals.")
        out.append(q)
        pos += q[3] + 1
    return out


def parse_gto(element, basis):
    """Per set: array (n_prim, 1 + n_contr) of alpha and coefficients (parse.py:143-176)."""
    ls = _lines(load_as_str(element, basis))
    quant = parse_quant_num(element, basis)
    out, pos = [], 4
    for q in quant:
        c = np.array([[float(v) for v in ls[pos + k].split()] for k in range(q[3])])
        if c.shape != (q[3], int(np.sum(q[4:])) + 1):
            raise ValueError(f"Line {ls[pos]} has incorrect number of coefficents.")
        out.append(c)
        pos += q[3] + 1
    return out


def _dfact(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def normalize_gto_coeff(quant_num, gto_coeffs):
    """Radially normalised contraction coefficients (parse.py:192-239)."""
    if len(quant_num) != len(gto_coeffs):
        raise ValueError("wrong coefficients for basis")
    out = []
    for q, c in zip(quant_num, gto_coeffs):
        a = c[:, 0]
        asum = a[:, None] + a[None, :]
        aprod = a[:, None] * a[None, :]
        cols = [c[:, 0:1]]
        col = 1
        for l in range(q[1], q[2] + 1):
            const = 2.0 ** (l + 1.75) / np.pi ** 0.25 / _dfact(2 * l + 1) ** 0.5
            for _ in range(q[4 + l - q[1]]):
                v = c[:, col]
                s = np.sum(np.outer(v, v) * asum ** (-l - 1.5) * aprod ** (l / 2 + 0.75))
                norm = (2.0 ** (l + 1.5) * s) ** -0.5
                cols.append((v * a ** (l / 2 + 0.75) * const * norm)[:, None])
                col += 1
        out.append(np.concatenate(cols, axis=1))
    return out


def basis_tables(basis):
    """AO table of one hydrogen for the engine.

    Returns (alpha[n_prim], coef[nao_atom, n_prim], l[nao_atom], cart[nao_atom]).
    AO order: every s contraction, then every p contraction as (x, y, z) --
    the order shared by the grid AOs (hqc/pbc/gto.py:268-288) and the analytic
    S/T blocks (hqc/pbc/solver.py:307-321) for sets that list s before p.
    Raises ValueError like the reference for l_min != 0 or l_max > 1
    (solver.py:83-86).
    """
    quant = parse_quant_num("H", basis)
    norm = normalize_gto_coeff(quant, parse_gto("H", basis))
    lmin = min(int(q[1]) for q in quant)
    lmax = max(int(q[2]) for q in quant)
    if lmin != 0:
        raise ValueError("l_min != 0")
    if lmax > 1:
        raise ValueError("l_max > 1 is not supported yet.")
    alpha = np.concatenate([c[:, 0] for c in norm])
    nprim = alpha.size
    rows, ls, carts = [], [], []
    off = 0
    seen_p = False
    for q, c in zip(quant, norm):
        col = 1
        for l in range(int(q[1]), int(q[2]) + 1):
            for _ in range(int(q[4 + l - q[1]])):
                full = np.zeros(nprim)
                full[off:off + c.shape[0]] = c[:, col]
                col += 1
                if l == 0:
                    if seen_p:
                        raise ValueError(f"basis {basis}: s contraction after a p contraction "
                                         "is not supported")
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
    return (np.ascontiguousarray(alpha), np.ascontiguousarray(np.array(rows)),
            np.array(ls, dtype=np.int32), np.array(carts, dtype=np.int32))
