"""Oracle frames in parallel host processes -- TEST INFRASTRUCTURE ONLY.

The restatement is single-threaded, like the reference.  Parity tests that
check many cloths, or frames in heavy contact (a 69 x 69 sheet draping a
sphere takes tens of seconds a frame), run the oracle's frames in a pool of
processes started with ``spawn`` (a process forked after the first CUDA call
would inherit a CUDA context it must not touch).

A job is ``(cloth, x, v, nframes, log, keep_every)``: the oracle cloth starts
from state (x, v) (None: its rest state), steps ``nframes`` frames of
``co_step`` (self_contact_sparse/main.cpp:213-263) and returns, for every
``keep_every``-th frame and the last one, ``(frame, x, v, contact_log, stats)``.
``contact_log`` lists the frame's detections as (kind, count, digest) when
``log`` is set (co_contact_log), else None.
"""
from __future__ import annotations

import multiprocessing as mp
import os

_LIB = {}


def _lib():
    from oracle import oracle as O
    if "port" not in _LIB:
        _LIB["port"] = O.OracleLib("port")
    return _LIB["port"]


def run_job(job):
    from oracle import oracle as O
    cloth, x, v, nframes, log, keep_every = job
    o = O.OracleCloth(_lib(), cloth)
    try:
        if x is not None:
            o.x[:] = x
            o.v[:] = v
        out = []
        for f in range(1, nframes + 1):
            if log:
                o.log_contacts(True)
            st = o.step(1)[0]
            if f == nframes or (keep_every and f % keep_every == 0):
                out.append((f, o.x.copy(), o.v.copy(), o.contact_log() if log else None, st))
        return out
    finally:
        o.close()


def run_jobs(jobs, processes: int | None = None, cost=None) -> list:
    """Runs the jobs in a spawn pool; results in job order.  ``cost`` (one
    number a job) orders the submissions, most expensive first."""
    from oracle import oracle as O
    O.build("port")
    jobs = list(jobs)
    if not jobs:
        return []
    n = processes or min(len(jobs), os.cpu_count() or 1)
    order = sorted(range(len(jobs)), key=lambda i: -(cost[i] if cost is not None else 0))
    with mp.get_context("spawn").Pool(n) as pool:
        pending = {i: pool.apply_async(run_job, (jobs[i],)) for i in order}
        return [pending[i].get() for i in range(len(jobs))]
