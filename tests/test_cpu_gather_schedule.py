"""The blocked layout's gather schedule (helm-project_gb300/csrc/
gather_schedule.hpp), compiled alone with g++ and checked on random warps
shaped like the headline's (rows of 3 to 17 entries over a block's few
hundred staged cells): every entry is read exactly once, by its own lane,
within the warp's steps; a lane's entries keep no required order but each
appears once; padding reads only the zero run; and the cost in shared-memory
wavefronts (per step, the most distinct addresses one bank holds) is below
that of a plain greedy order."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "helm-project_gb300", "csrc")


@pytest.fixture(scope="module")
def sched(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("sched") / "libsched.so")
    subprocess.run([gxx, "-std=c++20", "-O2", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(HERE, "native", "sched_harness.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    P = C.POINTER(C.c_int)
    lib.sched_warp.argtypes = [P, P, C.c_int, C.c_int, C.c_int, P, P]
    lib.sched_warp.restype = C.c_int
    return lib


def ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def wavefronts(q_steps):
    """Per step: the most distinct addresses any bank holds."""
    tot = 0
    for q in q_steps:
        banks = {}
        for a in set(int(v) for v in q):
            banks[a & 31] = banks.get(a & 31, 0) + 1
        tot += max(banks.values())
    return tot


def greedy_cost(rows, zero):
    """In-order reads (entry k of each row at step k, padding at the zero
    slot): the cost of an unscheduled layout."""
    W = max(len(r) for r in rows)
    steps = []
    for k in range(W):
        steps.append([r[k] if k < len(r) else zero for r in rows])
    return wavefronts(steps)


def random_warp(rng, n_cells=300):
    lens = np.sort(rng.integers(3, 18, 32))[::-1]
    rows = []
    for n in lens:
        c0 = rng.integers(0, n_cells - 24)
        rows.append(sorted(set(int(v) for v in c0 + rng.integers(0, 24, int(n) * 2)))[:int(n)])
    chunks = sorted(set(v >> 2 for r in rows for v in r))
    pos = {c: i for i, c in enumerate(chunks)}
    addr_rows = [[4 * pos[v >> 2] + (v & 3) for v in r] for r in rows]
    return addr_rows, 4 * len(chunks)


@pytest.mark.parametrize("seed", range(20))
def test_schedule_invariants_and_cost(sched, seed):
    rng = np.random.default_rng(seed)
    rows, zero = random_warp(rng)
    zrun = 32
    n_of = np.array([len(r) for r in rows], np.int32)
    addr = np.array([a for r in rows for a in r], np.int32)
    W = int(n_of.max())
    q = np.zeros(W * 32, np.int32)
    e = np.zeros(W * 32, np.int32)
    assert sched.sched_warp(ptr(n_of), ptr(addr), W, zero, zrun, ptr(q), ptr(e)) == 1
    q, e = q.reshape(W, 32), e.reshape(W, 32)
    starts = np.concatenate([[0], np.cumsum(n_of)])
    seen = np.zeros(len(addr), int)
    for k in range(W):
        for lane in range(32):
            if e[k, lane] < 0:
                assert zero <= q[k, lane] < zero + zrun  # padding reads the zero run only
            else:
                i = e[k, lane]
                assert starts[lane] <= i < starts[lane + 1]  # a lane reads its own row's entries
                assert q[k, lane] == addr[i]
                seen[i] += 1
    assert np.all(seen == 1)  # every entry exactly once
    assert wavefronts(q) < greedy_cost(rows, zero)


def test_shared_addresses_cost_one_wavefront(sched):
    # every lane's entries are the same four addresses in different banks:
    # a schedule exists with one wavefront per step
    rows = [[0, 1, 2, 3] for _ in range(32)]
    n_of = np.full(32, 4, np.int32)
    addr = np.array([a for r in rows for a in r], np.int32)
    q = np.zeros(4 * 32, np.int32)
    e = np.zeros(4 * 32, np.int32)
    assert sched.sched_warp(ptr(n_of), ptr(addr), 4, 4, 32, ptr(q), ptr(e)) == 1
    assert wavefronts(q.reshape(4, 32)) == 4


def test_empty_lanes_pad(sched):
    n_of = np.zeros(32, np.int32)
    n_of[0] = 2
    addr = np.array([5, 37], np.int32)  # one bank: they cannot share a step without conflict
    q = np.zeros(2 * 32, np.int32)
    e = np.zeros(2 * 32, np.int32)
    assert sched.sched_warp(ptr(n_of), ptr(addr), 2, 40, 32, ptr(q), ptr(e)) == 1
    e = e.reshape(2, 32)
    assert sorted(e[:, 0].tolist()) == [0, 1]
    assert np.all(e[:, 1:] == -1)
