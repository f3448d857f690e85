"""Admission of serving requests (physim_gb300/csrc/serve_admission.h), driven on the host.

The server admits a request when a slot is free and its device bytes fit the budget; the
instances it created stay resident while idle and count against the budget, and the least
recently used idle ones are evicted to make room.  A request larger than the whole budget
is refused.  These are the decisions phx_server_progress takes, through the same header.
"""
import ctypes as C

import numpy as np

ADMIT, WAIT_SLOTS, WAIT_MEMORY, EVICT, NEVER = range(5)


def decide(shim, active, slots, in_use, budget, need, residents=()):
    n = len(residents)
    b = np.array([r[0] for r in residents] or [0], dtype=np.int64)
    lu = np.array([r[1] for r in residents] or [0], dtype=np.uint64)
    idle = np.array([int(r[2]) for r in residents] or [0], dtype=np.int32)
    plan = np.zeros(max(1, n), dtype=np.int32)
    k = C.c_int()
    v = shim.adm_decide(active, slots, in_use, budget, need, n, b.ctypes.data, lu.ctypes.data, idle.ctypes.data,
                        plan.ctypes.data, C.byref(k))
    return v, list(plan[:k.value])


def test_request_larger_than_the_budget_is_refused(admission_shim):
    assert decide(admission_shim, 0, 4, 0, 100, 101)[0] == NEVER
    # even with every slot free and nothing resident
    assert decide(admission_shim, 0, 4, 0, 100, 100)[0] == ADMIT


def test_slots_before_memory(admission_shim):
    assert decide(admission_shim, 4, 4, 0, 100, 10)[0] == WAIT_SLOTS
    assert decide(admission_shim, 3, 4, 50, 100, 50)[0] == ADMIT


def test_waits_when_only_active_requests_hold_the_budget(admission_shim):
    # 90 bytes held by resident instances that are all busy: nothing can be evicted
    res = [(40, 1, False), (50, 2, False)]
    assert decide(admission_shim, 2, 8, 90, 100, 20, res) == (WAIT_MEMORY, [])


def test_evicts_least_recently_used_idle_instances_first(admission_shim):
    # idle instances used at ticks 5, 2, 9 (bytes 30, 30, 30) and one busy one
    res = [(30, 5, True), (30, 2, True), (30, 9, True), (10, 1, False)]
    # 100 of 120 in use; a 45-byte request needs 25 more: evict the oldest idle one (index 1)
    assert decide(admission_shim, 1, 8, 100, 120, 45, res) == (EVICT, [1])
    # a 75-byte request needs 55: the two oldest (1, then 0)
    assert decide(admission_shim, 1, 8, 100, 120, 75, res) == (EVICT, [1, 0])
    # 110 bytes: all three idle ones are not enough (only 90 freeable, 10 busy stays)
    assert decide(admission_shim, 1, 8, 100, 120, 111, res) == (WAIT_MEMORY, [])


def test_admission_sequence_keeps_the_budget(admission_shim):
    """A stream of requests against a 1000-byte budget: the in-use total never exceeds the
    budget, and every request that fits the budget is eventually admitted."""
    rng = np.random.default_rng(3)
    budget, slots = 1000, 3
    residents = {}  # id -> [bytes, last_used, idle]
    active = []
    tick = 0
    admitted = 0
    for rid in range(300):
        need = int(rng.integers(50, 400))
        for _ in range(50):
            in_use = sum(r[0] for r in residents.values())
            assert in_use <= budget
            ids = list(residents)
            v, plan = decide(admission_shim, len(active), slots, in_use, budget, need,
                             [tuple(residents[i]) for i in ids])
            if v in (ADMIT, EVICT):
                for k in plan:
                    assert residents[ids[k]][2]  # only idle instances are evicted
                    del residents[ids[k]]
                tick += 1
                residents[rid] = [need, tick, False]
                active.append(rid)
                admitted += 1
                break
            # finish the oldest active request (it stays resident, idle)
            assert v in (WAIT_SLOTS, WAIT_MEMORY) and active
            done = active.pop(0)
            tick += 1
            residents[done][1] = tick
            residents[done][2] = True
    assert admitted == 300
