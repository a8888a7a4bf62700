"""Many independent realisations on one GPU.

A disorder average (for example many random-field realisations of a tree
Hamiltonian) is a set of independent time evolutions. ``run_realisations``
advances them with several worker threads: each owns a CUDA stream and a share
of the realisations, builds their drivers on that stream and steps them.
Realisations never exchange data. The library's foreign calls and the stream
synchronisations release the interpreter lock, so GPU work of one realisation
can overlap host work of another; when the drivers' Python work dominates
(small trees), the interpreter lock serialises the workers and they run no
faster than one.
"""
from __future__ import annotations

import contextlib
import threading
from typing import Any, Callable

import torch

from . import _lib


def run_realisations(make: Callable[[int], Any], count: int, steps: int, workers: int = 4,
                     on_done: Callable[[int, Any], Any] | None = None, device: str | None = None) -> list:
    """Build realisation i with ``make(i)`` (a TDVP/TEBD driver), run ``steps``
    calls of ``run_one_time_step`` on it, and keep ``on_done(i, driver)`` (the
    driver itself by default). Realisation i runs on worker i mod ``workers``;
    the result list is in realisation order. Raises the first error any
    worker met."""
    _lib.load()
    use_streams = torch.cuda.is_available() and (device or "cuda") != "cpu" and _streams_available()
    results: list = [None] * count
    errors: list = []
    lock = threading.Lock()

    def work(wid: int):
        try:
            stream = torch.cuda.Stream() if use_streams else None
            ctx = torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext()
            with ctx:
                for i in range(wid, count, workers):
                    algo = make(i)
                    for _ in range(steps):
                        algo.run_one_time_step()
                    results[i] = on_done(i, algo) if on_done is not None else algo
                if stream is not None:
                    stream.synchronize()
        except BaseException as exc:     # surfaced to the caller below
            with lock:
                errors.append(exc)

    threads = [threading.Thread(target=work, args=(w,), daemon=True) for w in range(max(1, workers))]
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
