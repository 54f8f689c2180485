"""The server's admission policy (ctd_admission.h), compiled for the host
and driven through its failure paths with a fake allocator: arrival order
without overtaking, the slot limit, the memory budget (a job larger than
the budget runs alone), and an allocation failure that leaves the job
queued and the accounting untouched until a retry succeeds."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("adm") / "admission_host_check")
    subprocess.check_call([gxx, "-std=c++17", "-O1", "-Wall", "-o", exe, os.path.join(HERE, "admission_host_check.cpp")])
    return exe


def run(checker, script):
    out = subprocess.run([checker], input=script, capture_output=True, text=True, check=True).stdout
    return out.strip().split("\n")


def states(lines):
    return [tuple(map(int, ln.split())) for ln in lines if len(ln.split()) == 3 and not ln.startswith(("0 ", "-"))]


def test_budget_slots_and_order(checker):
    out = run(checker, "budget 100 max 3\nsubmit 40\nsubmit 50\nsubmit 20\nsubmit 5\nadmit\n")
    # 40 + 50 fit, 20 does not (110 > 100): admission stops there, 5 waits behind it
    assert out[-2] == "0 0 1" and out[-1] == "90 2 2"


def test_oversized_job_runs_alone(checker):
    out = run(checker, "budget 10 max 4\nsubmit 50\nsubmit 1\nadmit\nrelease 0\nadmit\n")
    assert out[-5] == "0 0" and out[-4] == "50 1 1"  # alone, beyond the budget
    assert out[-2] == "0 1" and out[-1] == "1 1 0"


def test_slot_limit(checker):
    out = run(checker, "budget 1000 max 2\nsubmit 1\nsubmit 1\nsubmit 1\nadmit\nrelease 1\nadmit\n")
    assert out[-5] == "0 0 1" and out[-4] == "2 2 1"
    assert out[-2] == "0 2" and out[-1] == "2 2 0"


def test_allocation_failure_keeps_job_queued(checker):
    out = run(checker, "budget 100 max 4\nsubmit 30\nsubmit 30\nadmit\nsubmit 30\nfail 1\nadmit\nadmit\n")
    assert out[3:5] == ["0 0 1", "60 2 0"]
    # the failed allocation: its status is returned, nothing is admitted or charged
    assert out[7:9] == ["-3", "60 2 1"]
    # the retry succeeds
    assert out[9:11] == ["0 2", "90 3 0"]
