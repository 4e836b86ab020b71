"""Host-side parsers against mutated inputs (tests/fuzz_host.py), each range
in a child process so that a crash fails the test instead of ending the
session: PNG and JPEG decoding, OBJ/MTL scene descriptions, the parameter
grammar, given trees. CPU only."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("kind,count", [("png", 10000), ("jpeg", 10000), ("obj", 10000), ("params", 10000),
                                        ("tree", 10000)])
def test_mutated_inputs_are_decoded_or_refused(kind, count):
    r = subprocess.run([sys.executable, os.path.join(HERE, "fuzz_host.py"), kind, "0", str(count)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, f"{kind}: exit {r.returncode}\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}"
    assert f"ok {kind} {count}" in r.stdout
