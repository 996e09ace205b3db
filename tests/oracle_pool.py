"""The float64 oracle's rayfunction over a process pool (test helper).

Large parity cases (1e6 rays) split their rays into interleaved chunks and
trace each chunk in its own process.  The pool uses ``spawn``: a forked
child of a process that has already used CUDA may hang.
"""

from __future__ import annotations

import concurrent.futures
import multiprocessing as mp
import os

import numpy as np


def _chunk(args):
    builder, kwargs, grid, exact = args
    from optika_gb300 import configs
    from oracle import trace as O

    system = getattr(configs, builder)(**kwargs)
    return O.rayfunction(system, grid["wavelength"], grid["field_x"], grid["field_y"],
                         grid["pupil_x"], grid["pupil_y"], exact=exact)


def rayfunction(builder: str, kwargs: dict, grid: dict, exact: bool = False,
                workers: int | None = None) -> dict:
    """``oracle.trace.rayfunction`` of ``configs.<builder>(**kwargs)`` on
    ``grid``, rays in their original order."""
    n = len(grid["wavelength"])
    workers = workers or max(1, min(16, len(os.sched_getaffinity(0))))
    parts = [{k: v[i::workers] for k, v in grid.items()} for i in range(workers)]
    ctx = mp.get_context("spawn")
    with concurrent.futures.ProcessPoolExecutor(max_workers=workers, mp_context=ctx) as ex:
        outs = list(ex.map(_chunk, [(builder, kwargs, p, exact) for p in parts]))
    ref = {}
    for k in outs[0]:
        a = np.empty(n, outs[0][k].dtype)
        for i in range(workers):
            a[i::workers] = outs[i][k]
        ref[k] = a
    return ref
