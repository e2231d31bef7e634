"""SQUANDER's own test files run unmodified against this package (CPU), where the reference tree
is present: its partitioning tests (tests/partitioning/test_partition.py) through the
`squander` alias of tests/reference_alias.py.  Deselected: the file's test that applies circuits
to states (it needs the GPU engine; its check, that the partitioned circuit computes the same
operator, is restated in tests/test_partition.py) and the one that builds CCX, CSWAP and SWAP
gates, which are outside the engine's gate set (the QASM reader expands them into it)."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SQG_REFERENCE_ROOT", "/root/reference")
PARTITION_TESTS = os.path.join(REF, "tests", "partitioning", "test_partition.py")


@pytest.mark.skipif(not os.path.exists(PARTITION_TESTS), reason="the reference tree is not present here")
def test_reference_partitioning_tests_pass_against_the_package(tmp_path):
    ini = tmp_path / "pytest.ini"
    ini.write_text("[pytest]\n")
    env = dict(os.environ, PYTHONPATH=HERE + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "pytest", PARTITION_TESTS, "-q", "-p", "reference_alias",
                        "-p", "no:cacheprovider", "-c", str(ini), "--rootdir", str(tmp_path),
                        "-k", "not CorrectnessOfPartitionedCircuit and not MaxQubitsEqualsTotalQubits"],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and " failed" not in r.stdout, r.stdout[-2000:]
