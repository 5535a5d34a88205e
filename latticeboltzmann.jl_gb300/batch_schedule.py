"""Which members of a DeviceBatch step block-resident, and on how many CTAs.

A batch member either takes the graph path (one kernel per global step, lbm_batch.cuh) or, when
it is small, the block-resident path (all of its steps of a call in one launch on a thread-block
cluster, lbm_resident.cuh).  Both give the same bits; the choice is speed only.  The choice is
read from ``batch_schedule.json`` beside this file, a table measured on the GPU by
``tune_batch.py`` (per storage and velocity set: the largest member that is faster resident, and
the nodes per CTA and the split of each node's collision over warps that were fastest there).  A
velocity set missing from the table takes the graph path.
"""
from __future__ import annotations

import json
import os

from . import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "batch_schedule.json")
QUAD_NAMES = ("D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21", "D2Q37")

_table = None


def measured_table():
    """The committed table {storage: {velocity set: {"resident_max_nodes", "nodes_per_block"}}}."""
    global _table
    if _table is None:
        with open(TABLE_PATH) as fh:
            _table = json.load(fh)
    return _table


def schedule_struct(rows):
    """An LbmBatchSchedule from {velocity set: {"resident_max_nodes": n, "nodes_per_block": p, "split": w}}
    ("split", the warps sharing a node's collision, defaults to 1)."""
    s = N.LbmBatchSchedule()
    for q, name in enumerate(QUAD_NAMES):
        row = rows.get(name) or {}
        s.resident_max_nodes[q] = int(row.get("resident_max_nodes", 0))
        s.nodes_per_block[q] = int(row.get("nodes_per_block", 0))
        s.split[q] = int(row.get("split", 1))
    return s


def schedule_for(storage, schedule="measured"):
    """The schedule a batch of `storage` members gets: "measured" (the table), None (every member
    on the graph path), or an explicit {velocity set: {...}} mapping."""
    if schedule is None:
        return None
    if schedule == "measured":
        return schedule_struct(measured_table().get("storages", {}).get(storage, {}))
    return schedule_struct(schedule)
