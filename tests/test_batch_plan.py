"""The batched gradient's per-job operation lists (seiswg_gb300/csrc/batch_plan.h,
the host logic of Batch's schedule) replayed on a model of each job's slots
for every step count up to 160, every checkpoint interval, both physics and
both recording modes, plus the configurations' sizes: every forward and
reverse step finds the state of its own step, checkpoints survive, the
reverse sweep runs nt-1 .. 0 with alternating adjoint slots.  Then the
launch plans of 3000 random mixes of jobs (plan_launches) under launch order
2 (a stream per kind and group, waits on the events of the kinds a launch's
jobs come from): by vector clocks, every job's operation at slot t comes
after its operation at slot t-1, and every wait is on a launch of slot t-1.
Binomial checkpointing (job_ops_revolve): its closed-form cost against a
brute-force minimisation, and its operation lists for nt up to 120 with 1 to
12 slots and the configurations' sizes replayed on the slots, recomputing
exactly the optimal number of steps.  The device queue of launch order 3
(plan_queue): 1500 random mixes run by a discrete-event model of the queue
kernel's warps (claiming units in order, waiting on the per-chunk counters)
with every unit's reads and writes, at the rows the marches really touch,
checked against each job's sequential order, and no deadlock.  A single
problem's recording pass (record_plan, Sim::forward_op) for every nt up to 160
and every interval: every launch reads the state of its step, checkpoints and
the final state hold theirs, and with every state kept the two-step launches
store the state between their steps.  The program
first shows that it reports planted mistakes (a dropped dependency bit, a
queue dependency that does not cover the rows read, a unit queued ahead of
its dependency).  CPU only (g++)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_job_operation_lists_replay_on_the_slots(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "batch_plan_check")
    src = os.path.join(ROOT, "tests", "batch_plan_check.cpp")
    inc = os.path.join(ROOT, "seiswg_gb300", "csrc")
    b = subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", f"-I{inc}", src, "-o", exe],
                       capture_output=True, text=True, timeout=300)
    assert b.returncode == 0, b.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    f = r.stdout.split()
    assert f[0] == "ok" and int(f[1]) > 50000 and int(f[2]) >= 3000 and int(f[3]) >= 2900 and int(f[4]) >= 1500
