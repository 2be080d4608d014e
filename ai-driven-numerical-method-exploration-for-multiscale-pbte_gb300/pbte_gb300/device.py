"""Stream-level synchronisation for the solve paths.

A solve waits only on the stream it runs on (the caller's current stream),
never on the whole device, so several solves can run side by side on their
own streams (:mod:`pbte_gb300.batch`)."""
from __future__ import annotations

import torch

__all__ = ["sync"]


def sync(device=None) -> None:
    """Wait for the work queued so far on the current stream of ``device``."""
    torch.cuda.current_stream(device).synchronize()
