"""siminf_gb300: SimInf's ssm/mssm Gillespie solver and scheduled-event engine
on one GB300 GPU, behind a C ABI (include/siminf_gb300.h) that replaces the
reference's SimInf_run_solver_ssm / SimInf_run_solver_mssm."""
from . import abi, model
from .model import SEIR, SIR, SIS, SISe, SISe3, SIR_mparse, SISe_pf, SimInfModel, make_events
from .abi import SimInfError

__all__ = ["abi", "model", "SimInfModel", "SIR", "SEIR", "SIS", "SISe", "SIR_mparse",
           "SISe_pf", "make_events", "SimInfError", "run", "pfilter", "prevalence",
           "individual_events"]


def run(*args, **kwargs):
    from .run import run as _run
    return _run(*args, **kwargs)


def pfilter(*args, **kwargs):
    from .run import pfilter as _pf
    return _pf(*args, **kwargs)


# trajectory() stays in siminf_gb300.trajectory: a package-level function of
# that name would be replaced by the submodule when it is imported.
def prevalence(*args, **kwargs):
    from .trajectory import prevalence as _prev
    return _prev(*args, **kwargs)


def individual_events(*args, **kwargs):
    from .individual import individual_events as _ie
    return _ie(*args, **kwargs)
