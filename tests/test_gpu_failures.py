"""Failure paths of a count, made on the host (no GPU fault): an interrupt signal between
launches (utils/macros.h:145-167: SIGTERM / SIGINT / SIGHUP abort the count with EXIT_FAILURE)
and a device / pinned allocation that fails (injected by CF_TEST_FAIL_ALLOC).  Each runs in a
child process: the failed call must return an error with a message, the next call must give the
right counts, and the caller's own signal handling must be back in place."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, signal, sys
import numpy as np
sys.path.insert(0, %(root)r)
from corrfunc_gb300 import theory
rng = np.random.default_rng(5)
x, y, z = (rng.random(20000) * 100.0 for _ in range(3))
bins = np.logspace(-1, np.log10(15.0), 10)
outcomes = []
for k in range(2):
    try:
        r = theory.DD(1, 1, bins, x, y, z, periodic=True, boxsize=100.0)
        outcomes.append(" ".join(str(int(v)) for v in r["npairs"]))
    except RuntimeError:
        outcomes.append("failed")
print("|".join(outcomes))
try:
    os.kill(os.getpid(), signal.SIGINT)
    for _ in range(1000):
        pass
    print("no KeyboardInterrupt")
except KeyboardInterrupt:
    print("KeyboardInterrupt")
"""


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    out = subprocess.run([sys.executable, "-c", CHILD % {"root": ROOT}], capture_output=True, text=True, env=env,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    return out.stdout.strip().split("\n"), out.stderr


@pytest.fixture(scope="module")
def expected():
    lines, _ = _run({})
    first, second = lines[0].split("|")
    assert first == second and first != "failed"
    return first


def test_interrupt_between_launches_fails_the_call_then_recovers(expected):
    lines, err = _run({"CF_TEST_SIGNAL": "1"})
    first, second = lines[0].split("|")
    assert first == "failed"
    assert "interrupted by signal 2" in err
    assert second == expected
    # the caller's SIGINT handler (Python's) is restored after each call
    assert lines[1] == "KeyboardInterrupt"


@pytest.mark.parametrize("nth", [1, 3, 7, 12])
def test_failed_allocation_fails_the_call_then_recovers(expected, nth):
    lines, err = _run({"CF_TEST_FAIL_ALLOC": str(nth)})
    first, second = lines[0].split("|")
    assert first == "failed"
    assert "injected by CF_TEST_FAIL_ALLOC" in err
    assert second == expected
