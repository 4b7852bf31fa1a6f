"""GB300-native engine for AeroKinetic's D3Q27 cumulant lattice-Boltzmann step.

Drop-in for the reference's uniform-grid CPU path: the same case classes
(Section, Flow, Grid, Plan, Project) and Solver interface, with the lattice
resident in GB300 HBM and every step executed by hand-written sm_103a kernels.
"""
from .geometry import Contour, Section, naca0012, naca4, naca4_parametric
from .config import Atmosphere, Flow, Grid, Plan
from .project import Project, RunSettings, StopCriteria

__version__ = "0.5.3+gb300"
__all__ = ["Contour", "Section", "naca0012", "naca4", "naca4_parametric", "Atmosphere", "Flow", "Grid", "Plan",
           "Project", "RunSettings", "StopCriteria", "Solver", "NumericalFailure", "build"]


def __getattr__(name):
    if name in ("Solver", "NumericalFailure"):
        from . import solver
        return getattr(solver, name)
    if name == "build":
        from ._native import build
        return build
    raise AttributeError(name)
