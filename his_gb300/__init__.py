"""GB300-native time step of the coupled 1-D/2-D flood engine.

Drop-in classes with the reference's engine interface (``SWE2D``, ``SWE1D``,
``exchange``, ``CoupledEngine``, ``MassBalance``) run every time step as
hand-written sm_103a CUDA kernels behind the C-ABI library ``libhis_gb300.so``
(``include/his_gb300.h``).  Importing the package does not load the library; the
first solver object does, and it raises if the library is missing.
"""
from .boundaries import EDGES, EdgeBC, all_edges, edge_values  # noqa: F401
from .config import SolverConfig  # noqa: F401
from .massbalance import TERMS, MassBalance  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    if name in ("SWE2D", "StepVolumes"):
        from . import swe2d
        return getattr(swe2d, name)
    if name in ("SWE1D", "Step1DVolumes", "Sections"):
        from . import swe1d
        return getattr(swe1d, name)
    if name in ("exchange", "CoupledEngine", "Links", "build_links", "NumericalInstabilityError"):
        from . import coupling
        return getattr(coupling, name)
    raise AttributeError(name)
