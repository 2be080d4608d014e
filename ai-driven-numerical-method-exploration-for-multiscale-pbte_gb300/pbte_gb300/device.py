"""Stream-level synchronisation for the solve paths, and the lock that keeps
device-wide operations out of CUDA graph captures.

A solve waits only on the stream it runs on (the caller's current stream),
never on the whole device, so several solves can run side by side on their
own streams (:mod:`pbte_gb300.batch`, :mod:`pbte_gb300.serve`).

Capturing a graph on one thread fails if another thread meanwhile makes a
device-wide synchronising call (context creation and destruction
synchronise and free device memory; a capture itself starts with a device
synchronisation).  Every capture and every such call therefore runs under
``device_lock``; kernel launches, copies and graph replays on a solve's own
stream do not take it."""
from __future__ import annotations

import threading

import torch

__all__ = ["sync", "device_lock", "bury", "empty_graveyard"]

#: held around graph captures and device-wide synchronising calls
device_lock = threading.RLock()

# CUDA graphs whose owner went away: destroying a graph while another thread
# captures invalidates that capture, so they wait here until a thread that
# holds device_lock empties the list
_graveyard: list = []


def bury(*graphs) -> None:
    """Keep graphs alive until :func:`empty_graveyard`."""
    _graveyard.extend(g for g in graphs if g is not None)


def empty_graveyard() -> None:
    """Destroy the buried graphs (the caller holds device_lock)."""
    _graveyard.clear()


def sync(device=None) -> None:
    """Wait for the work queued so far on the current stream of ``device``."""
    torch.cuda.current_stream(device).synchronize()
