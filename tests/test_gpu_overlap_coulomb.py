"""Standalone make_overlap (hqc/pbc/overlap.py) and the walker-batched
potential_energy (hqc/pbc/potential.py:69-101) against the reference's golden
values and the oracle.

Tolerances: S 1e-12 (the same FP64 lattice sums); Coulomb sums 1e-11 absolute
on the golden walkers and 1e-10 relative on large batches (the engine sums
the reciprocal part through structure factors, the reference pair by pair).
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("basis", ["gth-szv", "gth-dzv", "gth-dzvp"])
def test_make_overlap_matches_reference_golden(basis):
    from hqc_gb300 import make_overlap
    meta, z = load_golden("overlap")
    n, rs, L = meta["n"], meta["rs"], float(z["L"])
    tag = basis.replace("-", "_")
    for rcut in (18, 24):
        S = make_overlap(n, L, rs, basis, rcut=rcut)(z["xp"])
        np.testing.assert_allclose(_np(S), z[f"S_{tag}_{rcut}"], atol=1e-12)
    ov = make_overlap(n, L, rs, basis, gamma=False)
    Sk = ov(z["xp"], z["kpt"])
    assert Sk.dtype.is_complex
    np.testing.assert_allclose(_np(Sk), z[f"Sk_{tag}"], atol=1e-12)
    # batches over configurations and over k-points equal the single calls
    xs = np.stack([z["xp"], z["xp"] + 0.1])
    ks = np.stack([z["kpt"], -z["kpt"]])
    Sb = _np(ov(xs, ks))
    np.testing.assert_array_equal(Sb[0], _np(Sk))
    np.testing.assert_allclose(Sb[1], _np(ov(xs[1], ks[1])), atol=0)


def test_make_overlap_kinetic_matches_oracle():
    from hqc_gb300 import make_overlap
    from oracle.gpw import Setup
    meta, z = load_golden("overlap")
    n, rs, L = meta["n"], meta["rs"], float(z["L"])
    st = Setup(n, L, rs, "gth-dzvp", n_grid=5)
    for kpt in (None, z["kpt"]):
        S_ref, T_ref, _, _ = st.overlap_kinetic(z["xp"] * rs, kpt=kpt)
        if kpt is None:
            S, T = make_overlap(n, L, rs, "gth-dzvp").with_kinetic(z["xp"])
        else:
            S, T = make_overlap(n, L, rs, "gth-dzvp", gamma=False).with_kinetic(z["xp"], kpt)
        np.testing.assert_allclose(_np(S), S_ref, atol=1e-12)
        np.testing.assert_allclose(_np(T), T_ref, atol=1e-11)


def test_potential_energy_matches_reference_golden():
    from hqc_gb300 import potential_energy, kpoints, Madelung
    meta, z = load_golden("coulomb_pe")
    for tag, m in meta.items():
        G = kpoints(m["dim"], m["Gmax"])
        out = potential_energy(z["x_" + tag], m["kappa"], G, float(z["L_" + tag]), m["rs"])
        for v, k in zip(out, ("vpp", "vep", "vee")):
            np.testing.assert_allclose(_np(v), z[k + "_" + tag], atol=1e-11, err_msg=tag + k)
        assert abs(Madelung(m["dim"], m["kappa"], G) - float(z["madelung_" + tag])) < 1e-13


def test_potential_energy_large_batch_matches_oracle():
    """H54 walkers (54 protons + 54 electrons), Gmax 15: the structure-factor
    form against the pairwise oracle; the proton-proton part also equals
    potential_energy_pp minus its Madelung term."""
    from hqc_gb300 import potential_energy, kpoints, potential_energy_pp, Madelung
    from oracle.ewald import potential_energy as pe_ref
    n, rs = 54, 1.31
    L = (4 / 3 * np.pi * n) ** (1 / 3)
    rng = np.random.default_rng(12)
    x = rng.uniform(0, L, (24, 2 * n, 3))
    G = kpoints(3, 15)
    out = [_np(v) for v in potential_energy(x, 10.0, G, L, rs)]
    ref = pe_ref(x[:6], 10.0, G, L, rs)
    for v, r in zip(out, ref):
        np.testing.assert_allclose(v[:6], r, rtol=1e-10, atol=1e-10)
    # vpp here is 2 rs / L sum psi; potential_energy_pp is 2 / (L rs) sum psi + the Madelung term
    vpp_pp = float(potential_energy_pp(x[0, :n], L, rs))
    mad = n * Madelung(3, 10.0, G) / L / rs
    assert abs(out[0][0] / rs ** 2 - (vpp_pp - mad)) < 1e-9
