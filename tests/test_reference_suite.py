"""SQUANDER's own test files run unmodified against this package through the `squander` alias of
tests/reference_alias.py, where the reference tree is present (SQG_REFERENCE_ROOT, else the
reference's checkout path).

CPU: its partitioning tests (tests/partitioning/test_partition.py).  Deselected: the file's test
that applies circuits to states (it needs the GPU engine; its check, that the partitioned
circuit computes the same operator, is restated in tests/test_partition.py) and the one that
builds CCX, CSWAP and SWAP gates, which are outside the engine's gate set (the QASM reader
expands them into it).

GPU: its circuit tests (tests/gates/test_circuit.py: application to matrices, states and
rectangular slices, from the right, lists, gate fusion, derivatives, combined forward and
derivatives) and its adaptive-decomposer tests (tests/decomposition/
test_optmization_problem_combined.py: trace offset, Combined_Unitary, Batch, Grad).  Deselected
from the circuit tests: the float32 cases (the engine computes in FP64 only; the reference
itself disables float32 for its cost functions) and the cases that build H, X or GENERAL gates,
which are outside the engine's gate set."""
import os
import re
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SQG_REFERENCE_ROOT", "/root/reference")
PARTITION_TESTS = os.path.join(REF, "tests", "partitioning", "test_partition.py")
CIRCUIT_TESTS = os.path.join(REF, "tests", "gates", "test_circuit.py")
COMBINED_TESTS = os.path.join(REF, "tests", "decomposition", "test_optmization_problem_combined.py")
PARTITION_PASSED = 12
CIRCUIT_DESELECT = ("not f32 and not float32 and not noparams and not no_params and not general_operation "
                    "and not nested and not h_x")


def _run_reference_tests(tmp_path, files, select, expect):
    ini = tmp_path / "pytest.ini"
    ini.write_text("[pytest]\n")
    env = dict(os.environ, PYTHONPATH=HERE + os.pathsep + os.environ.get("PYTHONPATH", ""))
    cmd = [sys.executable, "-m", "pytest", *files, "-q", "-p", "reference_alias", "-p", "no:cacheprovider",
           "-c", str(ini), "--rootdir", str(tmp_path)]
    if select:
        cmd += ["-k", select]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " failed" not in r.stdout, r.stdout[-2000:]
    passed = re.search(r"(\d+) passed", r.stdout)
    assert passed and int(passed.group(1)) == expect, r.stdout[-2000:]


@pytest.mark.skipif(not os.path.exists(PARTITION_TESTS), reason="the reference tree is not present here")
def test_reference_partitioning_tests_pass_against_the_package(tmp_path):
    _run_reference_tests(tmp_path, [PARTITION_TESTS],
                         "not CorrectnessOfPartitionedCircuit and not MaxQubitsEqualsTotalQubits", PARTITION_PASSED)


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(CIRCUIT_TESTS), reason="the reference tree is not present here")
def test_reference_circuit_tests_pass_against_the_package(tmp_path):
    _run_reference_tests(tmp_path, [CIRCUIT_TESTS], CIRCUIT_DESELECT, 90)


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(COMBINED_TESTS), reason="the reference tree is not present here")
def test_reference_combined_problem_tests_pass_against_the_package(tmp_path):
    _run_reference_tests(tmp_path, [COMBINED_TESTS], None, 2)
