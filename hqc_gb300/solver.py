"""``make_solver``: the drop-in factory of hqc's periodic GPW SCF solver.

Same signature, argument meaning, units and return tuple as
``hqc/pbc/solver.py:14-32`` (inputs ``xp`` in rs units, outputs in Rydberg);
the work runs in the sm_103a engine behind ``include/hqcgb.h``.  Arrays come
back as float64 torch tensors on the GPU.  Extra keyword arguments:

* ``precision``: 'fp64' (plain double-precision path) or 'mixed'
  (tensor-core grid contractions, FP64 small linear algebra);
* ``forces``: keep what ``solver.grad`` needs for dE/dxp;
* ``n_grid``: override the grid size rule of solver.py:159.
"""
import ctypes
import weakref

import numpy as np
import torch

from . import _lib
from .basis import basis_tables

RY = 2.0
SEARCH = {"bisect": 0, "newton": 1}
SMEAR = {"fermi": 0, "gauss": 1}
PRECISION = {"fp64": 0, "mixed": 1}


def grid_size(L_bohr, grid_length):
    """Odd grid of the reference: round(L / grid_length / 2) * 2 + 1 (solver.py:159)."""
    return int(round(L_bohr / grid_length / 2)) * 2 + 1


def lattice_1d(L_bohr, rcut=24.0):
    """1D translations of the grid GTO sums (hqc/pbc/gto.py:47-49, rcut fixed at 24)."""
    tmax = rcut // L_bohr
    return np.arange(-tmax, tmax + 1) * L_bohr


def lattice_sphere(L_bohr, rcut):
    """Lattice vectors within rcut for the S/T sums (hqc/pbc/solver.py:162-176)."""
    tmax = rcut // L_bohr
    nt = np.arange(-tmax, tmax + 1)
    T = np.array(np.meshgrid(nt, nt, nt)).reshape(3, -1).T * L_bohr
    return np.ascontiguousarray(T[(T ** 2).sum(1) <= rcut ** 2])


def xc_code(xc):
    key = xc.lower().replace(" ", "")
    if key.split(",")[0] == "lda" and key.split(",")[1] in ("pz81", "pz"):
        # hqc/tools/excor.py:116-117 returns the undefined name pw91
        raise NameError("name 'pw91' is not defined")
    if key not in _lib.XC:
        if key.split(",")[0] not in ("lda", "pbe", "gga_x_pbe"):
            raise ValueError("exchange functional not supported yet.")
        raise ValueError("correlation functional not supported yet.")
    return _lib.XC[key]


def build_params(n, L_bohr, ng, basis, rcut, tol, max_cycle, diis, diis_space, diis_start_cycle,
                 diis_damp, dft, xc, smearing, smearing_method, smearing_sigma, search_method,
                 search_cycle, search_tol, precision, forces, exx_occ_threshold):
    """The engine's hqcgb_params for one system; returns (params, arrays the
    params point into, AOs per atom)."""
    alpha, coef, ls, carts = basis_tables(basis)
    lat1 = lattice_1d(L_bohr)
    lat = lattice_sphere(L_bohr, rcut)
    keep = [alpha, coef, ls, carts, lat1, lat]
    P = _lib.Params()
    P.n_atoms = n
    P.n_grid = ng
    P.L = L_bohr
    P.nao_atom = coef.shape[0]
    P.n_prim = alpha.size
    P.alpha = alpha.ctypes.data_as(_lib.c_double_p)
    P.coef = coef.ctypes.data_as(_lib.c_double_p)
    P.ao_l = ls.ctypes.data_as(_lib.c_int_p)
    P.ao_cart = carts.ctypes.data_as(_lib.c_int_p)
    P.n_lat1d = lat1.size
    P.lat1d = lat1.ctypes.data_as(_lib.c_double_p)
    P.n_lattice = lat.shape[0]
    P.lattice = lat.ctypes.data_as(_lib.c_double_p)
    P.dft = int(bool(dft))
    P.xc = xc_code(xc) if dft else 0
    P.smearing = int(bool(smearing))
    if smearing:
        assert smearing_method in SMEAR
        assert search_method in SEARCH
    P.smearing_method = SMEAR.get(smearing_method, 0)
    P.smearing_sigma = float(smearing_sigma)
    P.search_method = SEARCH.get(search_method, 0)
    P.search_cycle = int(search_cycle)
    P.search_tol = float(search_tol)
    P.tol = float(tol)
    P.max_cycle = int(max_cycle)
    P.diis = int(bool(diis))
    P.diis_space = int(diis_space)
    P.diis_start_cycle = int(diis_start_cycle)
    P.diis_damp = float(diis_damp)
    P.precision = PRECISION[precision]
    P.exx_occ_threshold = float(exx_occ_threshold)
    P.want_forces = int(bool(forces))
    return P, keep, coef.shape[0]


class Plan:
    """Owns one engine plan (device workspace for one system size)."""

    def __init__(self, n, L_bohr, basis, rcut, tol, max_cycle, grid_length, diis, diis_space,
                 diis_start_cycle, diis_damp, dft, xc, smearing, smearing_method, smearing_sigma,
                 search_method, search_cycle, search_tol, precision="fp64", forces=False,
                 n_grid=None, exx_occ_threshold=0.0, kpoint=False):
        lib = _lib.load()
        if not torch.cuda.is_available():
            raise RuntimeError("hqc_gb300 needs a CUDA GPU (no CPU fallback)")
        self.n = n
        self.L = L_bohr
        self.ng = grid_size(L_bohr, grid_length) if n_grid is None else int(n_grid)
        self.dft = bool(dft)
        P, self._keep, self.nao_atom = build_params(
            n, L_bohr, self.ng, basis, rcut, tol, max_cycle, diis, diis_space, diis_start_cycle,
            diis_damp, dft, xc, smearing, smearing_method, smearing_sigma, search_method,
            search_cycle, search_tol, precision, forces, exx_occ_threshold)
        self.nao = n * self.nao_atom
        self.params = P
        self.device = torch.device("cuda", torch.cuda.current_device())
        h = ctypes.c_void_p()
        self.kpoint = bool(kpoint)
        if self.kpoint:
            _lib.check(lib.hqcgb_kplan_create(ctypes.byref(P), ctypes.byref(h)))
            self._finalizer = weakref.finalize(self, lib.hqcgb_kplan_destroy, h)
        else:
            _lib.check(lib.hqcgb_plan_create(ctypes.byref(P), ctypes.byref(h)))
            self._finalizer = weakref.finalize(self, lib.hqcgb_plan_destroy, h)
        self.handle = h

    def stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def scf(self, xp_bohr):
        """Run the SCF at xp (Bohr, torch float64 (n, 3) on the device)."""
        lib = _lib.load()
        nao = self.nao
        dev = self.device
        out = dict(mo_coeff=torch.empty(nao, nao, dtype=torch.float64, device=dev),
                   dm=torch.empty(nao, nao, dtype=torch.float64, device=dev),
                   bands=torch.empty(nao, dtype=torch.float64, device=dev),
                   energies=torch.empty(5, dtype=torch.float64, device=dev),
                   converged=torch.zeros(1, dtype=torch.int32, device=dev),
                   iterations=torch.zeros(1, dtype=torch.int32, device=dev),
                   free_energy=torch.empty(1, dtype=torch.float64, device=dev))
        o = _lib.ScfOut(*[ctypes.c_void_p(out[k].data_ptr()) for k in
                          ("mo_coeff", "dm", "bands", "energies", "converged", "iterations",
                           "free_energy")])
        xp_bohr = xp_bohr.contiguous()
        st = lib.hqcgb_scf(self.handle, ctypes.c_void_p(xp_bohr.data_ptr()), ctypes.byref(o),
                           self.stream())
        _lib.check(st, allow=(0, 1))
        return out

    def scf_kpt(self, xps_bohr, kpts, forces=False):
        """k-point SCFs: xps_bohr (B, n, 3) on the device, kpts (B, 3) in
        1/Bohr (host array); mo_coeff and dm come back complex128.  With
        ``forces`` also "grad" (B, n, 3), dE/dR in Hartree/Bohr of each
        single-k free energy (hqcgb_pes_kpt_batch)."""
        lib = _lib.load()
        nao, dev = self.nao, self.device
        B = xps_bohr.shape[0]
        out = dict(mo_coeff=torch.empty(B, nao, nao, dtype=torch.complex128, device=dev),
                   dm=torch.empty(B, nao, nao, dtype=torch.complex128, device=dev),
                   bands=torch.empty(B, nao, dtype=torch.float64, device=dev),
                   energies=torch.empty(B, 5, dtype=torch.float64, device=dev),
                   converged=torch.zeros(B, dtype=torch.int32, device=dev),
                   iterations=torch.zeros(B, dtype=torch.int32, device=dev),
                   free_energy=torch.empty(B, dtype=torch.float64, device=dev))
        o = _lib.ScfOut(*[ctypes.c_void_p(out[k].data_ptr()) for k in
                          ("mo_coeff", "dm", "bands", "energies", "converged", "iterations",
                           "free_energy")])
        xps_bohr = xps_bohr.contiguous()
        k = np.ascontiguousarray(kpts, dtype=np.float64).reshape(B, 3)
        if forces:
            out["grad"] = torch.empty(B, self.n, 3, dtype=torch.float64, device=dev)
            st = lib.hqcgb_pes_kpt_batch(self.handle, B, ctypes.c_void_p(xps_bohr.data_ptr()),
                                         k.ctypes.data_as(_lib.c_double_p), ctypes.byref(o),
                                         ctypes.c_void_p(out["grad"].data_ptr()), self.stream())
        else:
            st = lib.hqcgb_scf_kpt_batch(self.handle, B, ctypes.c_void_p(xps_bohr.data_ptr()),
                                         k.ctypes.data_as(_lib.c_double_p), ctypes.byref(o), self.stream())
        _lib.check(st, allow=(0, 1))
        return out

    def forces_kpt(self):
        """dE/dR (Hartree/Bohr, (n, 3) on the device) of the last k-point SCF."""
        lib = _lib.load()
        g = torch.empty(self.n, 3, dtype=torch.float64, device=self.device)
        _lib.check(lib.hqcgb_forces_kpt(self.handle, ctypes.c_void_p(g.data_ptr()), self.stream()))
        return g

    def set_concurrency(self, workers):
        """Configurations a batch call runs at once (each extra one clones the
        workspace; see hqcgb_plan_set_concurrency)."""
        _lib.check(_lib.load().hqcgb_plan_set_concurrency(self.handle, int(workers)))

    def scf_batch(self, xps_bohr, forces=False, full=True):
        """SCF (and forces) of every configuration of xps_bohr (B, n, 3) on the
        device; full=False skips the per-configuration matrices."""
        lib = _lib.load()
        nao, dev = self.nao, self.device
        B = xps_bohr.shape[0]
        out = dict(bands=torch.empty(B, nao, dtype=torch.float64, device=dev),
                   energies=torch.empty(B, 5, dtype=torch.float64, device=dev),
                   converged=torch.zeros(B, dtype=torch.int32, device=dev),
                   iterations=torch.zeros(B, dtype=torch.int32, device=dev),
                   free_energy=torch.empty(B, dtype=torch.float64, device=dev))
        if full:
            out["mo_coeff"] = torch.empty(B, nao, nao, dtype=torch.float64, device=dev)
            out["dm"] = torch.empty(B, nao, nao, dtype=torch.float64, device=dev)
        ptr = lambda k: ctypes.c_void_p(out[k].data_ptr()) if k in out else ctypes.c_void_p(0)
        o = _lib.ScfOut(*[ptr(k) for k in ("mo_coeff", "dm", "bands", "energies", "converged",
                                            "iterations", "free_energy")])
        g = torch.empty(B, self.n, 3, dtype=torch.float64, device=dev) if forces else None
        xps_bohr = xps_bohr.contiguous()
        st = lib.hqcgb_pes_batch(self.handle, B, ctypes.c_void_p(xps_bohr.data_ptr()), ctypes.byref(o),
                                 ctypes.c_void_p(g.data_ptr() if g is not None else 0), self.stream())
        _lib.check(st, allow=(0, 1))
        out["grad"] = g
        return out

    def forces(self):
        """dE/dR (Hartree/Bohr) of the last SCF, (n, 3) on the device."""
        lib = _lib.load()
        g = torch.empty(self.n, 3, dtype=torch.float64, device=self.device)
        _lib.check(lib.hqcgb_forces(self.handle, ctypes.c_void_p(g.data_ptr()), self.stream()))
        return g

    def query(self, name):
        """An internal buffer as a flat float64 tensor (complex k-point
        matrices as interleaved pairs: ``torch.view_as_complex`` after a
        reshape to (..., 2))."""
        lib = _lib.load()
        q = lib.hqcgb_kplan_query if self.kpoint else lib.hqcgb_plan_query
        nbytes = q(self.handle, name.encode(), None, 0, self.stream())
        if nbytes < 0:
            raise KeyError(name)
        t = torch.empty(nbytes // 8, dtype=torch.float64, device=self.device)
        q(self.handle, name.encode(), ctypes.c_void_p(t.data_ptr()), nbytes, self.stream())
        return t


def _as_device(xp, device):
    if isinstance(xp, torch.Tensor):
        return xp.detach().to(device=device, dtype=torch.float64)
    return torch.as_tensor(np.asarray(xp, dtype=np.float64), device=device)


def make_solver(n: int, L: float, rs: float, basis: str,
                rcut: float = 24,
                tol: float = 1e-7,
                max_cycle: int = 100,
                grid_length: float = 0.12,
                diis: bool = True,
                diis_space: int = 8,
                diis_start_cycle: int = 1,
                diis_damp: float = 0.,
                use_jit: bool = True,
                dft: bool = False,
                xc: str = 'lda,vwn',
                smearing: bool = False,
                smearing_method: str = 'fermi',
                smearing_sigma: float = 0.,
                search_method: str = 'bisect',
                search_cycle: int = 100,
                search_tol: float = 1e-7,
                gamma: bool = True,
                precision: str = 'fp64',
                forces: bool = False,
                n_grid=None,
                exx_occ_threshold: float = 0.0,
                concurrency: int = 1):
    """PBC solver factory (hqc/pbc/solver.py:14-32).

    ``solver(xp)`` -> (mo_coeff, dm, bands, E, Ki, Vep, Vee, Se, converged):
    bands and energies in Rydberg, E excludes Vpp (solver.py:705-767).
    A batch xp of shape (B, n, 3) returns the same tuple with a leading batch
    axis -- what ``jax.vmap(solver)`` returns for the reference
    (test/test.py:157); ``concurrency`` configurations of a batch run at once.
    ``use_jit`` is accepted for signature compatibility (the engine is always
    compiled).

    ``gamma=False`` returns ``solver(xp, kpt)`` for one k-point (kpt (3,) in
    1/Bohr, first Brillouin zone (-pi/(L rs), pi/(L rs)); solver.py:769-962):
    the same tuple with complex128 mo_coeff and dm.
    ``precision='mixed'`` (Hartree-Fock and LDA) runs its grid contractions on
    the tensor cores (complex operands as real/imaginary rows, FP32 pair
    transforms) with the FP64 eigensolver; a batch of xp (B, n, 3) and/or kpt
    (B, 3) broadcasts like ``jax.vmap``.  With ``forces=True``,
    ``solver.grad()`` is the gradient (Rydberg per rs unit) of the last
    single-k call's free energy ``solver.free_energy`` and
    ``solver.batch(xp, kpt, forces=True)`` returns them per configuration.
    """
    L_bohr = float(L) * float(rs)
    if not gamma:
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"unknown precision {precision!r}")
        if precision == "mixed" and dft and _lib.XC.get(xc.lower().replace(" ", "")) == 10:
            raise NotImplementedError("the mixed k-point solver covers Hartree-Fock and LDA")
        return _make_kpoint_solver(n, L_bohr, rs, basis, rcut, tol, max_cycle, grid_length, diis,
                                   diis_space, diis_start_cycle, diis_damp, dft, xc, smearing,
                                   smearing_method, smearing_sigma, search_method, search_cycle,
                                   search_tol, n_grid, exx_occ_threshold, precision, forces)
    plan = Plan(n, L_bohr, basis, rcut, tol, max_cycle, grid_length, diis, diis_space,
                diis_start_cycle, diis_damp, dft, xc, smearing, smearing_method, smearing_sigma,
                search_method, search_cycle, search_tol, precision=precision, forces=forces,
                n_grid=n_grid, exx_occ_threshold=exx_occ_threshold)

    if concurrency > 1:
        plan.set_concurrency(concurrency)

    def batch(xps, forces=False, full=True):
        xp_t = _as_device(xps, plan.device)
        assert xp_t.dim() == 3 and xp_t.shape[1] == n
        out = plan.scf_batch(xp_t * rs, forces=forces, full=full)
        solver.iterations = out["iterations"].tolist()
        solver.free_energy = out["free_energy"] * RY
        return out

    def solver(xp):
        xp_t = _as_device(xp, plan.device)
        if xp_t.dim() == 3:
            out = batch(xp_t)
            e = out["energies"]
            return (out["mo_coeff"], out["dm"], out["bands"] * RY, e[:, 0] * RY, e[:, 1] * RY,
                    e[:, 2] * RY, e[:, 3] * RY, e[:, 4], out["converged"] != 0)
        assert xp_t.shape[0] == n
        out = plan.scf(xp_t * rs)
        e = out["energies"]
        solver.iterations = int(out["iterations"].item())
        solver.free_energy = out["free_energy"][0] * RY
        return (out["mo_coeff"], out["dm"], out["bands"] * RY, e[0] * RY, e[1] * RY, e[2] * RY,
                e[3] * RY, e[4], out["converged"][0] != 0)

    def grad(xp=None):
        """Gradient (Rydberg per rs unit) of the last call's free energy
        ``solver.free_energy`` = E - sigma S (E itself without smearing; S the
        entropy that makes the smeared occupations stationary); needs
        forces=True."""
        return plan.forces() * (RY * rs)

    solver.plan = plan
    solver.grad = grad
    solver.batch = batch
    solver.n_grid = plan.ng
    return solver


def _make_kpoint_solver(n, L_bohr, rs, basis, rcut, tol, max_cycle, grid_length, diis, diis_space,
                        diis_start_cycle, diis_damp, dft, xc, smearing, smearing_method,
                        smearing_sigma, search_method, search_cycle, search_tol, n_grid,
                        exx_occ_threshold, precision="fp64", forces=False):
    plan = Plan(n, L_bohr, basis, rcut, tol, max_cycle, grid_length, diis, diis_space,
                diis_start_cycle, diis_damp, dft, xc, smearing, smearing_method, smearing_sigma,
                search_method, search_cycle, search_tol, precision=precision, forces=forces,
                n_grid=n_grid, exx_occ_threshold=exx_occ_threshold, kpoint=True)

    def _broadcast(xp, kpt):
        xp_t = _as_device(xp, plan.device)
        k = np.asarray(kpt.detach().cpu() if isinstance(kpt, torch.Tensor) else kpt, dtype=np.float64)
        batched = xp_t.dim() == 3 or k.ndim == 2
        B = max(xp_t.shape[0] if xp_t.dim() == 3 else 1, k.shape[0] if k.ndim == 2 else 1)
        xps = xp_t.expand(B, n, 3) if xp_t.dim() == 3 else xp_t.reshape(1, n, 3).expand(B, n, 3)
        ks = np.broadcast_to(k.reshape(-1, 3), (B, 3))
        return xps.contiguous(), ks, batched

    def batch(xp, kpt, forces=False):
        """Every (xp, kpt) pair of the broadcast batch; with ``forces`` also
        "grad" (B, n, 3) in Rydberg per rs unit."""
        xps, ks, _ = _broadcast(xp, kpt)
        out = plan.scf_kpt(xps * rs, ks, forces=forces)
        solver.iterations = out["iterations"].tolist()
        solver.free_energy = out["free_energy"] * RY
        if forces:
            out["grad"] = out["grad"] * (RY * rs)
        return out

    def solver(xp, kpt):
        xps, ks, batched = _broadcast(xp, kpt)
        out = plan.scf_kpt(xps * rs, ks)
        solver.iterations = out["iterations"].tolist()
        solver.free_energy = out["free_energy"] * RY if batched else out["free_energy"][0] * RY
        e = out["energies"]
        res = (out["mo_coeff"], out["dm"], out["bands"] * RY, e[:, 0] * RY, e[:, 1] * RY,
               e[:, 2] * RY, e[:, 3] * RY, e[:, 4], out["converged"] != 0)
        if not batched:
            res = tuple(r[0] for r in res)
            solver.iterations = solver.iterations[0]
        return res

    def grad(xp=None):
        """Gradient (Rydberg per rs unit) of the last single-k call's free
        energy ``solver.free_energy``; needs forces=True."""
        return plan.forces_kpt() * (RY * rs)

    solver.plan = plan
    solver.grad = grad
    solver.batch = batch
    solver.n_grid = plan.ng
    return solver
