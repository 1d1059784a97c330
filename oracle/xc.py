"""Oracle exchange-correlation functionals.

LDA pieces restate ``hqc/tools/excor.py:3-126``: epsilon_x (Slater), and the
correlations '', vwn, hl71, bh72, gl77.  The reference obtains
v = eps + rho d eps / d rho with ``jax.grad`` per grid point
(``hqc/pbc/solver.py:672-678``); here the derivative is taken by the
complex-step method, exact to rounding for these analytic formulas.
'pz81' raises NameError as in the reference (excor.py:116-117 returns the
undefined name ``pw91``).

GGA-PBE is not in the reference (parity unpinned): PBE exchange and
correlation (Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996)) on top of the PW92
LDA correlation (Perdew & Wang, PRB 45, 13244 (1992)), spin-unpolarised.
Test infrastructure only.
"""
import numpy as np

WS = (3 / 4 / np.pi) ** (1 / 3)

# VWN (excor.py:37-49)
_A, _Y0, _B, _C = 0.0621814, -0.10498, 3.72744, 12.93532
_YY0 = _Y0 ** 2 + _B * _Y0 + _C
_Q = (4 * _C - _B ** 2) ** 0.5
_C0 = _A / 2
_C1 = _C0 * 2 * _B / _Q
_C2 = _C0 * _B * _Y0 / _YY0
_C3 = _C2 * 2 * (_B + 2 * _Y0) / _Q
_C4 = _C1 - _C3

_HL = {"hl": (21.0, 0.045), "hl71": (21.0, 0.045), "bh": (30.0, 0.0504),
       "bh72": (30.0, 0.0504), "gl": (11.4, 0.0666), "gl77": (11.4, 0.0666)}


def eps_x_lda(rho):
    return -3 / 4 * (3 / np.pi) ** (1 / 3) * rho ** (1 / 3)


def eps_vwn(rho):
    rs = WS / rho ** (1 / 3)
    y = np.sqrt(rs)
    Yy = y ** 2 + _B * y + _C
    atnp = np.arctan(_Q / (2 * y + _B))
    return _C0 * np.log(y ** 2 / Yy) + _C4 * atnp - _C2 * np.log((y - _Y0) ** 2 / Yy)


def eps_hl_family(rho, A, C):
    rs = WS / rho ** (1 / 3)
    x = rs / A
    return -0.5 * C * ((1 + x ** 3) * np.log(1 + 1 / x) + x / 2 - x ** 2 - 1 / 3)


# PBE ------------------------------------------------------------------------
_KAPPA = 0.804
_BETA = 0.06672455060314922
_MU = _BETA * np.pi ** 2 / 3
_GAMMA = (1 - np.log(2)) / np.pi ** 2
_PW = dict(A=0.0310907, a1=0.21370, b1=7.5957, b2=3.5876, b3=1.6382, b4=0.49294)


def eps_c_pw92(rs):
    p = _PW
    q = 2 * p["A"] * (p["b1"] * rs ** 0.5 + p["b2"] * rs + p["b3"] * rs ** 1.5 + p["b4"] * rs ** 2)
    return -2 * p["A"] * (1 + p["a1"] * rs) * np.log(1 + 1 / q)


def e_pbe(rho, sigma):
    """PBE energy per volume rho*eps_xc(rho, |grad rho|^2)."""
    kf = (3 * np.pi ** 2 * rho) ** (1 / 3)
    ex_unif = -3 * kf / (4 * np.pi)
    s2 = sigma / (4 * kf ** 2 * rho ** 2)
    Fx = 1 + _KAPPA - _KAPPA / (1 + _MU * s2 / _KAPPA)
    rs = (3 / (4 * np.pi * rho)) ** (1 / 3)
    ec = eps_c_pw92(rs)
    ks2 = 4 * kf / np.pi
    t2 = sigma / (4 * ks2 * rho ** 2)
    A = (_BETA / _GAMMA) / (np.exp(-ec / (_GAMMA)) - 1)
    At2 = A * t2
    H = _GAMMA * np.log(1 + (_BETA / _GAMMA) * t2 * (1 + At2) / (1 + At2 + At2 ** 2))
    return rho * (ex_unif * Fx + ec + H)


class Functional:
    """xc string as in ``make_solver(xc=...)``: 'lda,<corr>' or 'pbe'."""

    RHO_MIN = 1e-14  # below this density the point contributes nothing

    def __init__(self, xc):
        xc = xc.lower().strip()
        if xc in ("pbe", "gga_x_pbe,gga_c_pbe", "pbe,pbe"):
            self.gga = True
            self.kind = "pbe"
            return
        self.gga = False
        parts = xc.split(",")
        exch, corr = parts[0], parts[1]
        if exch != "lda":
            raise ValueError("exchange functional not supported yet.")
        if corr in ("pz81", "pz"):
            raise NameError("name 'pw91' is not defined")
        if corr not in ("", "vwn") and corr not in _HL:
            raise ValueError("correlation functional not supported yet.")
        self.kind = corr

    def eps(self, rho):
        e = eps_x_lda(rho)
        if self.kind == "vwn":
            e = e + eps_vwn(rho)
        elif self.kind in _HL:
            e = e + eps_hl_family(rho, *_HL[self.kind])
        return e

    def evaluate(self, rho, sigma=None):
        """Return (e, v_rho, v_sigma): energy per volume and its partials."""
        h = 1e-30
        if not self.gga:
            ec = self.eps(rho + 1j * h * rho)  # complex step, relative
            eps = ec.real
            deps = ec.imag / (h * rho)
            return rho * eps, eps + rho * deps, None
        ok = rho > self.RHO_MIN
        r = np.where(ok, rho, 1.0)
        s = np.where(ok, sigma, 0.0)
        e = e_pbe(r, s)
        vr = e_pbe(r + 1j * h * r, s).imag / (h * r)
        vs = e_pbe(r, s + 1j * h * np.maximum(s, 1e-30)).imag / (h * np.maximum(s, 1e-30))
        return (np.where(ok, e, 0.0), np.where(ok, vr, 0.0), np.where(ok, vs, 0.0))
