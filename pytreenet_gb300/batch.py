"""Many independent realisations on one GPU.

A disorder average (for example many random-field realisations of a tree
Hamiltonian) is a set of independent time evolutions. ``run_realisations``
advances them with worker threads, each owning a CUDA stream and a share of
the realisations, and optionally with several worker processes.
Realisations never exchange data.

Threads overlap one realisation's GPU work with another's host work: the
library's foreign calls and the stream synchronisations release the
interpreter lock. When the drivers' Python work dominates (small trees and
bond dimensions: about 0.4 s of host work per two-site step on the 31-site
binary tree), the lock serialises the threads and they run no faster than one.
Worker processes (``processes`` > 1, started with ``spawn``) each have their
own interpreter and CUDA context on the same GPU, so the host work runs in
parallel; their kernels share the GPU by time slicing.
"""
from __future__ import annotations

import contextlib
import multiprocessing
import threading
from typing import Any, Callable

import torch

from . import _lib


def run_realisations(make: Callable[[int], Any], count: int, steps: int, workers: int = 4,
                     on_done: Callable[[int, Any], Any] | None = None, device: str | None = None,
                     processes: int = 1, pool=None) -> list:
    """Build realisation i with ``make(i)`` (a TDVP/TEBD driver), run ``steps``
    calls of ``run_one_time_step`` on it, and keep ``on_done(i, driver)`` (the
    driver itself by default). The result list is in realisation order. Raises
    the first error any worker met.

    ``processes`` > 1 (or a ``pool`` from ``realisation_pool``) splits the
    realisations over worker processes, each running ``workers`` threads on
    its share (realisation i in process i mod ``processes``). ``make`` and
    ``on_done`` must then be picklable (module-level functions), and
    ``on_done`` is required: drivers stay in their process, only its results
    come back."""
    _lib.load()
    if pool is not None or processes > 1:
        if on_done is None:
            raise ValueError("run_realisations with worker processes needs on_done (drivers stay in their process)")
        nproc = getattr(pool, "_processes", processes) if pool is not None else processes
        chunks = [list(range(p, count, nproc)) for p in range(nproc)]
        tasks = [(make, idx, steps, workers, on_done, device) for idx in chunks if idx]
        own = pool is None
        if own:
            pool = realisation_pool(nproc)
        try:
            parts = pool.map(_process_share, tasks)
        finally:
            if own:
                pool.close()
                pool.join()
        results: list = [None] * count
        for (_, idx, *_rest), res in zip(tasks, parts):
            for i, r in zip(idx, res):
                results[i] = r
        return results
    return _run_threads(make, list(range(count)), steps, workers, on_done, device)


def realisation_pool(processes: int):
    """A pool of ``processes`` worker processes started with ``spawn`` (a fork
    of a process that has used CUDA would not work); keep it across calls of
    ``run_realisations(..., pool=pool)`` to pay the start-up (interpreter,
    library, CUDA context) once."""
    return multiprocessing.get_context("spawn").Pool(processes)


def _process_share(task):
    make, idx, steps, workers, on_done, device = task
    return _run_threads(make, idx, steps, workers, on_done, device)


def _run_threads(make, indices: list, steps: int, workers: int, on_done, device) -> list:
    use_streams = torch.cuda.is_available() and (device or "cuda") != "cpu" and _streams_available()
    results: list = [None] * len(indices)
    errors: list = []
    lock = threading.Lock()
    workers = max(1, workers)

    def work(wid: int):
        try:
            stream = torch.cuda.Stream() if use_streams else None
            ctx = torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext()
            with ctx:
                for j in range(wid, len(indices), workers):
                    i = indices[j]
                    algo = make(i)
                    for _ in range(steps):
                        algo.run_one_time_step()
                    results[j] = on_done(i, algo) if on_done is not None else algo
                if stream is not None:
                    stream.synchronize()
        except BaseException as exc:     # surfaced to the caller below
            with lock:
                errors.append(exc)

    threads = [threading.Thread(target=work, args=(w,), daemon=True) for w in range(workers)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return results


def _streams_available() -> bool:
    try:
        return torch.cuda.device_count() > 0
    except Exception:
        return False
