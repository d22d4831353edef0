"""C-ABI checks that need no GPU: the library builds, loads and exports every
entry point include/swm_gpu.h declares; configuration errors that are
detected before any device work come back as error codes."""
import ctypes
import os
import re

import pytest

from cubedsphere_sbp_swm_gb300 import _abi, build as swm_build
import cubedsphere_sbp_swm_gb300 as swm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "swm_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(swm_[a-z0-9_]+)\s*\(", text)))


def test_header_matches_binding_table():
    assert _declared() == sorted(_abi.EXPORTS)


def test_library_exports_every_declared_symbol():
    path = swm_build.build()
    lib = ctypes.CDLL(path)
    missing = [name for name in _declared() if not hasattr(lib, name)]
    assert not missing, missing


@pytest.mark.parametrize("names,code", [
    (dict(div_op_name="divergence_c_sbp42"), _abi.SWM_E_UNSUPPORTED),
    (dict(grad_op_name="gradient_ah63_sbp_ecs"), _abi.SWM_E_UNSUPPORTED),   # mixed orders
    (dict(coriolis_op_name="coriolis_Cgrid_sbp42"), _abi.SWM_E_UNSUPPORTED),
    (dict(quadrature_name="SBP_C42_quadrature"), _abi.SWM_E_UNSUPPORTED),
])
def test_unknown_operator_names_are_rejected(names, code):
    base = dict(div_op_name="divergence_ah42_sbp", grad_op_name="gradient_ah42_sbp_ecs",
                curl_op_name="curl_divergence_ah42_sbp", coriolis_op_name="coriolis_colocated",
                KE_op_name="KE_colocated", co2contra_op_name="co2contra_colocated",
                massflux_op_name="massflux_colocated", quadrature_name="SBP_Ah42_quadrature")
    base.update(names)
    with pytest.raises(swm.SwmError) as e:
        swm.OperatorSWM(swm.ModelConfig(N=32, names=base))
    assert e.value.code == code


def test_bad_sizes_are_rejected():
    with pytest.raises(swm.SwmError) as e:
        swm.OperatorSWM(swm.ModelConfig(N=4))
    assert e.value.code == _abi.SWM_E_INVALID
    with pytest.raises(swm.SwmError) as e:
        swm.OperatorSWM(swm.ModelConfig(N=32, sbp_order=21))
    assert e.value.code == _abi.SWM_E_UNSUPPORTED


def test_unknown_time_scheme_and_halo():
    assert isinstance(swm.create_timescheme("explicit_Eul1"), swm.ExplicitEul1)
    with pytest.raises(swm.SwmError):
        swm.create_timescheme("ars343")
    with pytest.raises(swm.SwmError):
        swm.create_halo_procedure(None, "ECS_O")
