"""CPU-side checks of the product: the C-ABI library loads and exports every
symbol declared in include/hqcgb.h; the basis parser and the host tables
match the oracle.  No GPU compute is called here."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "hqcgb.h")).read()
    return sorted(set(re.findall(r"\b(hqcgb_[a-z_]+)\s*\(", text)))


def test_header_symbols_exported():
    from hqc_gb300 import build, _lib
    build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 9
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(_lib.EXPORTS)


def test_last_error_and_bad_args_without_gpu():
    from hqc_gb300 import _lib
    lib = _lib.load()
    P = _lib.Params()
    P.n_atoms = 0
    h = ctypes.c_void_p()
    st = lib.hqcgb_plan_create(ctypes.byref(P), ctypes.byref(h))
    assert st == 2  # HQCGB_BAD_ARG, validated before any device call
    assert b"n_atoms" in lib.hqcgb_last_error()
    # the k-point force entry points refuse null plans and outputs the same way
    assert lib.hqcgb_forces_kpt(None, None, None) == 2
    assert b"null" in lib.hqcgb_last_error()
    out = _lib.ScfOut()
    assert lib.hqcgb_pes_kpt_batch(None, 1, None, None, ctypes.byref(out), None, None) == 2
    assert b"null" in lib.hqcgb_last_error()


@pytest.mark.parametrize("basis", ["gth-szv", "gth-dzv", "gth-dzvp", "gth-tzv2p", "gth-qzv2p"])
def test_basis_tables_match_oracle(basis):
    from hqc_gb300.basis import basis_tables
    from oracle.basis import Basis
    a, c, l, cart = basis_tables(basis)
    B = Basis(basis)
    np.testing.assert_allclose(a, B.alpha, rtol=0, atol=0)
    np.testing.assert_allclose(c, B.coef, rtol=1e-14, atol=1e-15)
    assert list(l) == list(B.l) and list(cart) == list(B.cart)


def test_basis_errors_like_reference():
    from hqc_gb300.basis import basis_tables, load_as_str
    with pytest.raises(ValueError):
        basis_tables("gth-cc-tzvp")  # d functions: l_max > 1 (solver.py:85-86)
    with pytest.raises(FileNotFoundError):
        load_as_str("H", "no-such-basis")


def test_grid_and_lattice_rules():
    from hqc_gb300.solver import grid_size, lattice_1d, lattice_sphere
    from oracle.gpw import Setup
    for n, rs, gl in [(4, 1.5, 0.12), (8, 1.25, None), (54, 1.31, None)]:
        L = (4 / 3 * np.pi * n) ** (1 / 3)
        gl = gl or L * rs / 80
        st = Setup(n, L, rs, "gth-szv", grid_length=gl)
        assert grid_size(L * rs, gl) == st.ng
        np.testing.assert_array_equal(lattice_1d(L * rs), st.lat1d)
        assert lattice_sphere(L * rs, 24.0).shape == st.lattice.shape


def test_xc_codes_and_reference_errors():
    from hqc_gb300.solver import xc_code
    assert xc_code("lda,vwn") == 1 and xc_code("pbe") == 10
    with pytest.raises(NameError):
        xc_code("lda,pz81")
    with pytest.raises(ValueError):
        xc_code("b3lyp,x")


def test_ewald_host_helpers_match_oracle():
    """kpoints / Madelung (hqc/pbc/potential.py:6-33) of the package against
    the oracle, 3D and 2D, and the simple-cubic Madelung known answer."""
    from hqc_gb300.potential import kpoints, Madelung
    from oracle.ewald import kpoints as kp_ref, madelung_dim
    for dim, gmax in ((3, 15), (3, 4), (2, 10)):
        G = kpoints(dim, gmax)
        ref = kp_ref(dim, gmax)
        assert G.shape == ref.shape
        assert sorted(map(tuple, G)) == sorted(map(tuple, ref))
        assert abs(Madelung(dim, 10.0, G) - madelung_dim(dim, 10.0, ref)) < 1e-13
    assert abs(Madelung(3, 10.0, kpoints(3, 15)) - (-2.8372974794806)) < 1e-9


def test_kpoint_factories_reject_unsupported_modes():
    """make_solver(gamma=False) has no mixed PBE path (with or without
    forces); the factories refuse it (and unknown precisions) before any
    device work."""
    from hqc_gb300 import make_solver, make_pes
    with pytest.raises(NotImplementedError):
        make_solver(4, 2.5, 1.5, "gth-szv", gamma=False, precision="mixed", dft=True, xc="pbe")
    with pytest.raises(ValueError):
        make_solver(4, 2.5, 1.5, "gth-szv", gamma=False, precision="half")
    with pytest.raises(NotImplementedError):
        make_pes(4, 2.5, 1.5, "gth-szv", gamma=False, forces=True, precision="mixed", dft=True, xc="pbe")


def test_overlap_lattice_sphere_matches_reference_rule():
    """The lattice sphere of make_overlap / the S, T sums: integer multiples
    of L within rcut (hqc/pbc/overlap.py:126-138, solver.py:162-176)."""
    from hqc_gb300.solver import lattice_sphere
    L = 3.7
    for rcut in (18.0, 24.0):
        T = lattice_sphere(L, rcut)
        tmax = rcut // L
        n = np.arange(-tmax, tmax + 1)
        ref = np.array(np.meshgrid(n, n, n)).reshape(3, -1).T * L
        ref = ref[(ref ** 2).sum(1) <= rcut ** 2]
        assert sorted(map(tuple, np.round(T / L).astype(int))) == sorted(map(tuple, np.round(ref / L).astype(int)))


def test_complex_diis_solve_matches_numpy():
    """The k-point DIIS coefficients (host code of the library, no GPU): the
    reference's unconjugated complex B (scf.py:177-188) with its eta
    regularisation, against numpy.linalg.solve of the same bordered system;
    the coefficients sum to 1."""
    from hqc_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(3)
    for sp in (1, 3, 8):
        e = rng.normal(size=(sp, 6, 6)) + 1j * rng.normal(size=(sp, 6, 6))
        B = np.einsum("imn,jmn->ij", e, e)  # complex symmetric, no conjugation
        eta = 1e-12 * (np.trace(B) / sp + 1.0)
        h = np.zeros((sp + 1, sp + 1), complex)
        h[:sp, :sp] = B + eta * np.eye(sp)
        h[:sp, sp] = -1
        h[sp, :sp] = -1
        g = np.zeros(sp + 1, complex)
        g[sp] = -1
        ref = np.linalg.solve(h, g)[:sp]
        Bi = np.ascontiguousarray(np.stack([B.real, B.imag], -1).reshape(-1))
        out = np.zeros(2 * sp)
        assert lib.hqcgb_diis_coefficients(sp, Bi.ctypes.data_as(_lib.c_double_p),
                                           out.ctypes.data_as(_lib.c_double_p)) == 0
        c = out[0::2] + 1j * out[1::2]
        np.testing.assert_allclose(c, ref, rtol=1e-9, atol=1e-12)
        assert abs(c.sum() - 1) < 1e-10


@pytest.mark.parametrize("nao", [1, 14, 16, 17, 20, 54, 127, 128, 129, 140, 144, 150, 256, 257, 270,
                                 300, 384, 400, 512, 513, 600, 900, 912, 913, 1000, 1024])
@pytest.mark.parametrize("sym", [True, False])
def test_quadrature_tile_plan_covers_each_tile_once(nao, sym):
    """The tensor-core quadrature's tile plan (host code of the library, no
    GPU): every destination tile of M (the upper triangle when symmetric) is
    written by exactly one product; each product's operand rows match its
    tile (transposed products swap them; the corner reads the narrow block on
    both sides); the MMA N covers the rows of the B-side block in multiples of
    16; the persistent form is taken exactly when there are 1..6 full blocks,
    the last block has at most 16 rows (or there is none), and not for one
    full block plus a partial one in the non-symmetric case (its only tile
    would need both orientations); the tile-list kernel gets at most 12 tiles
    per launch."""
    from hqc_gb300 import _lib
    tiles, launches = _lib.quad_tiles(nao, sym)
    nblk = -(-nao // 128)
    last = nao - 128 * (nblk - 1)
    narrow = last < 128
    nfull = nblk - 1 if narrow else nblk
    cover = np.zeros((nblk, nblk), int)
    for kind, mt, nt, arow, brow, nb, swap in tiles:
        assert 0 <= mt < nblk and 0 <= nt < nblk
        cover[mt, nt] += 1
        a_blk, b_blk = (nt, mt) if swap else (mt, nt)
        assert (arow, brow) == (128 * a_blk, 128 * b_blk)
        b_rows = min(128, nao - brow)
        assert nb % 16 == 0 and b_rows <= nb <= 128, (kind, mt, nt, nb)
        if kind == 1:
            assert nb == 16 and b_blk == nblk - 1
    want = np.triu(np.ones((nblk, nblk), int)) if sym else np.ones((nblk, nblk), int)
    np.testing.assert_array_equal(cover, want)
    persist = (last <= 16 or not narrow) and 1 <= nfull <= 6 and not (nfull == 1 and narrow and not sym)
    assert (tiles[:, 0] != 2).any() == persist
    n_list = int((tiles[:, 0] == 2).sum())
    assert launches == int(persist) + -(-n_list // 12)
    if persist:
        assert n_list == 0
        # one narrow product per tile of the partial block: (m, last) for
        # every full block m, (last, n) too when not symmetric, and the corner
        assert int((tiles[:, 0] == 1).sum()) == (0 if not narrow else (nfull + 1 if sym else 2 * nfull + 1))


def test_autograd_wrapper_chains_engine_gradient():
    """The torch.autograd.Function over value_and_grad (host logic only): a
    stand-in pes with E = sum x^3 per configuration and its exact gradient;
    torch.autograd must return dE/dxp times the incoming gradient, for one
    configuration and for a batch."""
    import torch
    from hqc_gb300 import pes_energy

    class FakePes:
        calls = 0

        def value_and_grad(self, xp):
            FakePes.calls += 1
            x = torch.as_tensor(xp, dtype=torch.float64)
            return (x ** 3).sum(dim=(-2, -1)), 3 * x ** 2

    pes = FakePes()
    x1 = torch.randn(4, 3, dtype=torch.float64, requires_grad=True)
    (g1,) = torch.autograd.grad(2.5 * pes_energy(x1, pes), x1)
    torch.testing.assert_close(g1, 7.5 * x1.detach() ** 2)
    xb = torch.randn(3, 4, 3, dtype=torch.float64, requires_grad=True)
    w = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64)
    E = pes_energy(xb, pes)
    assert E.shape == (3,)
    (gb,) = torch.autograd.grad((w * E).sum(), xb)
    torch.testing.assert_close(gb, w[:, None, None] * 3 * xb.detach() ** 2)
    assert FakePes.calls == 2  # one engine call per forward, none in backward

    class FakeKpes:
        def value_and_grad(self, xp, kpt):
            x = torch.as_tensor(xp, dtype=torch.float64)
            k = torch.as_tensor(kpt, dtype=torch.float64).reshape(-1, 3)[:, 0]
            E = (x ** 3).sum(dim=(-2, -1)) * (1 + k)
            g = 3 * x ** 2 * (1 + k)[:, None, None]
            return (E[0], g[0]) if torch.as_tensor(kpt).dim() == 1 else (E, g)

    kp = FakeKpes()
    (gk,) = torch.autograd.grad(pes_energy(x1, kp, [0.5, 0.0, 0.0]), x1)
    torch.testing.assert_close(gk, 1.5 * 3 * x1.detach() ** 2)
    mesh = torch.tensor([[0.0, 0, 0], [1.0, 0, 0]], dtype=torch.float64)
    Em = pes_energy(x1, kp, mesh)
    assert Em.shape == (2,)
    (gm,) = torch.autograd.grad(Em.sum(), x1)  # both k-points act on the same positions
    torch.testing.assert_close(gm, (1.0 + 2.0) * 3 * x1.detach() ** 2)



def test_pes_host_logic_with_stand_in_engine(monkeypatch):
    """make_pes's host logic (pes.py:78-137 of the reference) over stand-ins
    for the engine calls: E + Vpp in 'default' mode, the 7-tuple in 'dev'
    mode, batches and nested-list inputs, the Gamma / k-point call forms and
    the reference's mode error."""
    import torch
    from hqc_gb300 import pes as pes_mod

    def fake_make_solver(n, L, rs, basis, gamma=True, **kw):
        def solver(xp, *kpt):
            x = torch.as_tensor(xp, dtype=torch.float64)
            E = x.sum(dim=(-2, -1)) + (float(kpt[0][0]) if kpt else 0.0)
            one = torch.ones_like(E)
            return None, None, None, E, 2 * one, 3 * one, 4 * one, 5 * one, one > 0

        def batch(xp, forces=False, full=True):
            x = torch.as_tensor(xp, dtype=torch.float64)
            # engine outputs in Hartree; the free energy differs from E (smearing)
            return {"energies": torch.stack([x.sum(dim=(-2, -1)) / 2.0] * 5, -1), "grad": x / 2.0,
                    "free_energy": x.sum(dim=(-2, -1)) / 2.0 - 0.25}

        solver.batch = batch
        solver.grad = lambda: None
        return solver

    def fake_vpp(xp, L, rs, kappa=10, Gmax=15):
        x = torch.as_tensor(xp, dtype=torch.float64)
        return 100.0 * x.shape[0] * torch.ones((), dtype=torch.float64), torch.full_like(x, 7.0)

    monkeypatch.setattr(pes_mod, "make_solver", fake_make_solver)
    monkeypatch.setattr(pes_mod, "potential_energy_pp_and_grad", fake_vpp)
    with pytest.raises(ValueError, match="Invalid mode"):
        pes_mod.make_pes(2, 2.0, 1.3, "gth-szv", mode="bad")
    xp = [[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]]
    pes = pes_mod.make_pes(2, 2.0, 1.3, "gth-szv")
    assert abs(float(pes(xp)) - (2.1 + 200.0)) < 1e-12
    xb = [xp, [[1.0, 0.0, 0.0], [0.0, 0.0, 0.0]]]
    np.testing.assert_allclose(pes(xb).numpy(), [202.1, 201.0])
    with pytest.raises(TypeError):
        pes(xp, np.zeros(3))
    dev = pes_mod.make_pes(2, 2.0, 1.3, "gth-szv", mode="dev")(xp)
    assert len(dev) == 7 and abs(float(dev[4]) - 200.0) < 1e-12 and float(dev[1]) == 2.0
    # batch: the engine's free energy (the gradient's own function) in Ha -> Ry,
    # gradients per rs unit
    E, g = pes.value_and_grad(xb)
    np.testing.assert_allclose(E.numpy(), [2.1 - 0.5 + 200.0, 1.0 - 0.5 + 200.0])
    np.testing.assert_allclose(g.numpy(), np.asarray(xb) / 2.0 * 2.0 * 1.3 + 7.0)
    kp = pes_mod.make_pes(2, 2.0, 1.3, "gth-szv", gamma=False)
    assert abs(float(kp(xp, np.array([0.5, 0.0, 0.0]))) - (2.6 + 200.0)) < 1e-12
    with pytest.raises(TypeError):
        kp(xp)


def test_kpoint_value_and_grad_host_logic(monkeypatch):
    """pes.value_and_grad(xp, kpt) over a stand-in k-point engine: one
    configuration at one k-point gives a scalar and an (n, 3) gradient; a
    k-mesh or a batch of configurations gives a leading batch axis, with
    the Ewald term of each configuration (expanded over the mesh when one
    configuration is shared); the free energy comes back in Rydberg and the
    Gamma-point call form is refused."""
    import torch
    from hqc_gb300 import pes as pes_mod

    def fake_make_solver(n, L, rs, basis, gamma=True, **kw):
        assert gamma is False and kw.get("forces")

        def batch(xp, kpt, forces=False):
            x = torch.as_tensor(xp, dtype=torch.float64)
            k = np.asarray(kpt, dtype=np.float64).reshape(-1, 3)
            B = max(x.shape[0] if x.dim() == 3 else 1, k.shape[0])
            xs = x.expand(B, n, 3) if x.dim() == 3 else x.reshape(1, n, 3).expand(B, n, 3)
            kk = torch.as_tensor(np.broadcast_to(k, (B, 3))[:, 0].copy())
            # Hartree free energies; gradients already in Ry per rs unit
            return {"free_energy": xs.sum(dim=(-2, -1)) / 2.0 + kk, "grad": xs + kk[:, None, None]}

        def solver(xp, kpt):
            raise AssertionError("value_and_grad goes through solver.batch")

        solver.batch = batch
        return solver

    def fake_vpp(xp, L, rs, kappa=10, Gmax=15):
        x = torch.as_tensor(xp, dtype=torch.float64)
        return 100.0 * x.shape[0] * torch.ones((), dtype=torch.float64), torch.full_like(x, 7.0)

    monkeypatch.setattr(pes_mod, "make_solver", fake_make_solver)
    monkeypatch.setattr(pes_mod, "potential_energy_pp_and_grad", fake_vpp)
    pes = pes_mod.make_pes(2, 2.0, 1.3, "gth-szv", gamma=False, forces=True)
    xp = np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]])
    F, g = pes.value_and_grad(xp, np.array([0.5, 0.0, 0.0]))
    assert F.dim() == 0 and g.shape == (2, 3)
    assert abs(float(F) - ((2.1 / 2.0 + 0.5) * 2.0 + 200.0)) < 1e-12
    np.testing.assert_allclose(g.numpy(), xp + 0.5 + 7.0)
    mesh = np.array([[0.1 * k, 0.0, 0.0] for k in range(8)])
    F, g = pes.value_and_grad(torch.as_tensor(xp), mesh)
    assert F.shape == (8,) and g.shape == (8, 2, 3)
    np.testing.assert_allclose(F.numpy(), (2.1 / 2.0 + mesh[:, 0]) * 2.0 + 200.0)
    xb = np.stack([xp, xp + 1.0])
    F, g = pes.value_and_grad(xb, np.zeros(3))
    assert F.shape == (2,) and g.shape == (2, 2, 3)
    np.testing.assert_allclose(F.numpy(), [2.1 + 200.0, 8.1 + 200.0])
    with pytest.raises(TypeError):
        pes.value_and_grad(xp)


def test_no_cpu_fallback(monkeypatch, tmp_path):
    """The product path fails loudly instead of falling back to CPU code:
    without the built library the loader raises, and without a GPU the
    factories raise before any work."""
    import torch
    from hqc_gb300 import _lib, make_solver, make_overlap
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load()
    monkeypatch.undo()
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError, match="CUDA GPU"):
            make_solver(2, 2.0, 1.5, "gth-szv")
        with pytest.raises(Exception):
            make_overlap(2, 2.0, 1.5, "gth-szv")(np.zeros((2, 3)))


def test_plain_c_client_links_and_runs(tmp_path):
    """tests/c_client.c, a C99 program using only include/hqcgb.h, compiles
    with gcc, links against the library and gets the expected answers from
    the host-side entry points (no GPU needed)."""
    import shutil
    import subprocess
    from hqc_gb300 import _lib
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    _lib.load()
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "c_client")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_client.c"),
                    "-L", libdir, "-lhqcgb", "-Wl,-rpath," + libdir, "-lm", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert "c_client ok" in r.stdout


def test_jax_ffi_handler_matches_its_python_wrapper():
    """The XLA FFI handlers (hqc_gb300/jax_ffi/pes_ffi.cc, compiled only where
    jaxlib is installed) and the ffi_calls in hqc_gb300/jax_ffi/__init__.py
    agree on the call signature: the same attribute names, as many results
    as the wrapper declares, two positional arguments at the Gamma point and
    three (with the k-points) for the single-k form."""
    import re
    src = open(os.path.join(ROOT, "hqc_gb300", "jax_ffi", "pes_ffi.cc")).read()
    py = open(os.path.join(ROOT, "hqc_gb300", "jax_ffi", "__init__.py")).read()
    n_out = py[py.index("def _outs("):py.index("def _finish(")].count("ShapeDtypeStruct(")
    for symbol, target, n_args in (("HqcgbPes", "hqcgb_pes", 2), ("HqcgbPesKpt", "hqcgb_pes_kpt", 3)):
        start = src.index(f"XLA_FFI_DEFINE_HANDLER_SYMBOL({symbol},")
        bind = src[start:src.index(");", start)]
        attrs = re.findall(r'\.Attr<[^>]+>\("(\w+)"\)', bind)
        assert attrs == ["plan", "L_rs", "rs", "kappa", "gmax"]
        for a in attrs:
            assert re.search(rf"\b{a}=np\.", py), a
        assert len(re.findall(r"\.Ret<", bind)) == n_out == 6
        assert len(re.findall(r"\.Arg<", bind)) == n_args
        assert f'"{target}"' in py and f"lib.{symbol})" in py
    # the handlers' results are the ABI's outputs: the PES batches + hqcgb_ewald
    hdr = open(os.path.join(ROOT, "include", "hqcgb.h")).read()
    for fn in ("hqcgb_pes_batch", "hqcgb_pes_kpt_batch", "hqcgb_ewald", "hqcgb_last_error"):
        assert fn in src and fn in hdr


def test_tuning_knobs_and_cache(monkeypatch, tmp_path):
    """Host side of the autotuner: knobs set and read back through the C ABI
    (no GPU work), unknown knobs rejected, and a measured choice cached per
    key so that a second run applies it without measuring."""
    from hqc_gb300 import tune, _lib
    tune.set_knob("quad_kchunk", 4096)
    assert tune.get_knob("quad_kchunk") == 4096
    tune.set_knob("quad_kchunk", 0)
    assert tune.get_knob("quad_kchunk") == 0
    with pytest.raises(_lib.HqcgbError):
        tune.set_knob("no_such_knob", 1)
    monkeypatch.setattr(tune, "CACHE", str(tmp_path / "tune.json"))
    calls = []

    def measure():
        calls.append(1)
        return 8192, {2048: 2.0, 8192: 1.0}

    assert tune._cached("gpu|quad_kchunk|270|81", measure) == (8192, {2048: 2.0, 8192: 1.0})
    assert tune._cached("gpu|quad_kchunk|270|81", measure) == (8192, None)
    assert len(calls) == 1
