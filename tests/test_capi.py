"""The C ABI library: builds, loads, exports every entry point that
include/siminf_gb300.h declares, and keeps the argument struct
layout-identical to the reference's SimInf_solver_args.  No GPU needed."""
import ctypes as C
import os
import re

import pytest

from siminf_gb300 import abi, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "siminf_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^(?:int|void|long long)\s+(siminf_gpu_\w+)\s*\(", text,
                                 re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "siminf_gpu_run_solver_ssm" in names
    assert "siminf_gpu_run_solver_mssm" in names
    assert set(names) == set(native.EXPORTS)


def test_library_builds_and_exports_every_symbol():
    from siminf_gb300 import build
    path = build.build()
    lib = C.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_args_struct_matches_c_layout(oracle_lib):
    # oracle_args_size() is sizeof(siminf_gpu_solver_args) from the C compiler;
    # ref_driver.c static-asserts it equals sizeof(SimInf_solver_args).
    assert oracle_lib.lib().oracle_args_size() == C.sizeof(abi.SolverArgs)
    assert abi.SolverArgs.seed.offset % 8 == 0


def test_no_device_is_an_error_not_a_fallback():
    """Without a GPU the library refuses to run (no CPU fallback)."""
    import numpy as np
    from siminf_gb300 import model as M
    from siminf_gb300.run import run
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    m = M.SIR_mparse({"S": [10], "I": [1], "R": [0]}, np.arange(1, 5), 0.1, 0.1)
    with pytest.raises(abi.SimInfError) as e:
        run(m)
    assert e.value.code == -34
