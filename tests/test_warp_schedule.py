"""Structure of the warp integrator's generated programs (csrc/gen/gen_warp.py), independent of numerics.

The interpreter runs a level's instructions on different lanes at once and meets between levels, and
the slot allocator reuses slots by liveness.  For every surface model's grad and energy programs:
  * a level holds instructions of one kind, at most as many as the group has lanes;
  * every operand is a constant, an input or the result of an earlier level;
  * no slot is written while a value it holds is still to be read (a later reader sees its own value);
  * the program's outputs are never overwritten after they are produced;
  * sums have 1..3 terms, and a term keeps a sign only when both factors are variables (the others were
    folded into negated constants);
  * every committed record of generated/warp_prog.h encodes exactly these instructions."""
import os
import re
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GEN = os.path.join(ROOT, "coarseair_gb300", "csrc", "gen")
sys.path.insert(0, GEN)

import gen_warp  # noqa: E402

TABS = None


def _model(key):
    global TABS
    if TABS is None:
        import json
        TABS = json.load(open(os.path.join(ROOT, "coarseair_gb300", "csrc", "generated", "pip_tables.json")))
    return gen_warp.compile_model(key, TABS)


@pytest.mark.parametrize("key", list(gen_warp.MODELS))
def test_levels_respect_dependencies_and_slot_lifetimes(key):
    m = _model(key)
    lanes = m["lanes"]
    for name in ("grad", "energy"):
        p = m["progs"][name]
        ins, slot, levels = p["ins"], p["slot"], p["levels"]
        level_of = {n: L for L, (_, nodes) in enumerate(levels) for n in nodes}
        nconst = m["nconst"]
        inputs = set(p["ins_slots"])
        writes = {}   # slot -> list of (level, node)
        for L, (kind, nodes) in enumerate(levels):
            assert 1 <= len(nodes) <= lanes
            assert all(ins[n][0] == kind for n in nodes)
            for n in nodes:
                writes.setdefault(slot[n], []).append((L, n))
                for x in gen_warp.operands(ins, n):
                    if x in level_of:
                        assert level_of[x] < L, (key, name, "operand produced at the same or a later level")
                    else:
                        s = slot[x]
                        assert s < nconst or s in inputs, (key, name, "operand neither constant, input nor computed")
                if kind == "sop":
                    terms = ins[n][1]
                    assert 1 <= len(terms) <= 3
                    for sg, a, b in terms:
                        if sg < 0:
                            for f in (a, b):
                                assert f in level_of or slot[f] in inputs, (key, name, "sign left on a constant factor")
        # liveness: between a value's write and its last read, no other write to its slot
        for L, (kind, nodes) in enumerate(levels):
            for n in nodes:
                for x in gen_warp.operands(ins, n):
                    if x not in level_of:
                        continue
                    w = level_of[x]
                    for (Lw, other) in writes[slot[x]]:
                        assert not (w < Lw <= L and other != x), (key, name, "slot overwritten before its last read")
        for o in p["out_nodes"]:
            later = [Lw for (Lw, other) in writes[slot[o]] if Lw > level_of[o]]
            assert not later, (key, name, "an output is overwritten after it is produced")
        assert p["nslot"] <= m["nslot"] and all(slot[n] < m["nslot"] for n in level_of)


def _records(text, key, name):
    g = re.search(r"wp_%s_%s_rec\[\d+\] __attribute__\(\(aligned\(16\)\)\) = \{([^}]*)\}" % (key, name), text)
    return np.array([int(x) for x in g.group(1).split(",")], dtype=np.uint64).reshape(-1, 8)


@pytest.mark.parametrize("key", list(gen_warp.MODELS))
def test_committed_records_encode_the_schedule(key):
    m = _model(key)
    text = open(os.path.join(ROOT, "coarseair_gb300", "csrc", "generated", "warp_prog.h")).read()
    lanes = m["lanes"]
    for name in ("grad", "energy"):
        p = m["progs"][name]
        rec = _records(text, key, name)
        ref = np.array(gen_warp.records(p["levels"], p["ins"], p["slot"], lanes, m["zero"]), dtype=np.uint64).reshape(-1, 8)
        assert np.array_equal(rec, ref)
        meta = rec[:, 0]
        active = (meta >> 31) & 1
        assert int(active.sum()) == sum(len(nodes) for _, nodes in p["levels"])
        # level-uniform kind, term count and sign flag
        for L in range(len(rec) // lanes):
            blk = meta[L * lanes:(L + 1) * lanes]
            on = blk[((blk >> 31) & 1) == 1]
            assert len(set(((on >> 23) & 0xFF).tolist())) == 1
