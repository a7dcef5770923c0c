"""Flag handling of the command-line driver (nns_gb300/nbx_runner), on the CPU:
the reference's main.cu flags are parsed before any CUDA call, so help,
unknown flags, missing values, empty runs and unknown models are answered
without a GPU (exit 0 for help, 2 for a usage error)."""
import subprocess

import pytest


@pytest.fixture(scope="module")
def runner():
    from nns_gb300 import build
    build.build()
    return build.RUNNER


def _run(runner, *args):
    return subprocess.run([runner, *args], capture_output=True, text=True, timeout=60)


def test_help(runner):
    out = _run(runner, "-h")
    assert out.returncode == 0 and "[-i iterations]" in out.stdout and "--model" in out.stdout


@pytest.mark.parametrize("args,msg", [
    (("--no-such-flag",), "unknown option --no-such-flag"),
    (("-i",), "missing value for -i"),
    (("-n", "10", "--model"), "missing value for --model"),
    (("--model", "spiral"), "unknown model spiral"),
    (("-n", "0"), ""),
    (("-i", "0"), ""),
])
def test_usage_errors(runner, args, msg):
    out = _run(runner, *args)
    assert out.returncode == 2, (args, out.stdout, out.stderr)
    assert msg in out.stderr
