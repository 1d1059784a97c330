"""GB300-native (sm_103a) periodic GPW SCF engine with hqc's Python API.

Drop-in factories: ``make_solver``, ``make_lcao``, ``make_pes`` (Gamma
and single k-point), ``make_slater``, ``make_overlap``, and the Ewald sums
``potential_energy_pp`` / ``potential_energy`` (reference: ZihangL/hqc
``hqc/pbc``); ``make_pes_batch`` runs configurations of uneven size in one
call.  The compute
runs in ``libhqcgb.so`` (``include/hqcgb.h``); there is no CPU fallback.
"""
from .solver import make_solver  # noqa: F401
from .lcao import make_lcao  # noqa: F401
from .pes import make_pes  # noqa: F401
from .potential import (potential_energy_pp, potential_energy_pp_and_grad,  # noqa: F401
                        potential_energy, kpoints, Madelung)
from .overlap import make_overlap  # noqa: F401
from .slater import make_slater  # noqa: F401
from .autograd import PesFunction, pes_energy  # noqa: F401
from .batch import make_pes_batch  # noqa: F401
from . import basis  # noqa: F401

__version__ = "0.1.0"
