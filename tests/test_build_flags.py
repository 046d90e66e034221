"""The compile flags the bit-identical FP64 results rest on (no GPU needed).

Every CUDA unit with FP64 arithmetic that must round like the oracle is built
without FMA contraction; that includes the mixed-precision unit, whose
dataflow sweep runs the FP64 Newton update that k_update runs in rc_core.cu.
The mixed unit gets its fast FP32 math from named SFU intrinsics, not from
--use_fast_math (which would also contract FP64 a*b+c).  The oracle and the
host set-up are built with -ffp-contract=off.
"""
import os
import re

from rocketcombustor_gb300 import build

import oracle


def test_cuda_units_do_not_contract_fp64():
    for unit, flags in build.UNITS.items():
        assert "--use_fast_math" not in flags, unit
        if unit != "rc_mlp.cu":  # BF16/FP32 network only
            assert "--fmad=false" in flags, unit


def test_mixed_unit_calls_the_sfu_math_by_name():
    src = open(os.path.join(build.CSRC, "rc_thermo32.cuh")).read()
    assert not re.search(r"(?<![_\w])(expf|logf|powf)\(", src)
    assert "__expf(" in src and "__logf(" in src
    assert {"--prec-div=false", "--prec-sqrt=false", "--ftz=true"} <= set(build.UNITS["rc_mixed.cu"])


def test_host_and_oracle_do_not_contract():
    assert any("-ffp-contract=off" in f for f in build.NVCC_COMMON)  # host code of the CUDA units
    assert "-ffp-contract=off" in oracle.CXXFLAGS
