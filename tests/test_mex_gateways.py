"""The model and solver MEX gateways (mex/msot_model_mex.cpp,
rec_nn_with_L2_reg.cpp, rec_nn_with_L1_eye_reg.cpp, rec_nn_with_TV_reg.cpp)
compile against the MEX API (the project's stand-in header here, MATLAB's
mex.h on a MATLAB host) and reject bad arguments before any device work;
the GPU runs of the same gateways are in test_gpu_mex_gateways.py."""
import ctypes as C

import pytest

import mexdrv


@pytest.fixture(scope="module")
def drv(tmp_path_factory):
    from msot_gb300 import _lib
    _lib.load(build_if_missing=True)  # the gateways link the library
    return mexdrv.build(str(tmp_path_factory.mktemp("mexdrv")))


@pytest.mark.parametrize("case,err_id", [
    (0, "msot_model_mex:command"),
    (1, "msot_model_mex:field"),
    (2, "rec_nn_with_L2_reg:model"),
    (3, "rec_nn_with_L1_eye_reg:model"),
])
def test_gateway_argument_errors(drv, case, err_id):
    msg = C.create_string_buffer(512)
    assert drv.drv_error_case(case, msg, 512) == 1
    assert msg.value.decode().split("|")[0] == err_id
    # no model was created, so the MEX file is not locked
    assert drv.drv_lock_count() == 0
