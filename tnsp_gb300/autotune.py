"""Per-lattice launch tuning of the sampler.

The sampler kernel runs one chain per thread block; how many blocks share an SM trades concurrency
(chains in flight, latency hiding) against the shared memory each block gets for staging the charge
sectors of its factorisations (sectors that do not fit are staged in the block's HBM slot).  The best
split depends on the lattice: its bond dimension, cut and sector sizes.  ``tune_blocks_per_sm`` times
the candidates on the lattice itself and keeps the fastest (TNSP_OPT_BLOCKS_PER_SM).

The probe is ``tnsp_amplitude`` (the row-0 strip: one down boundary per row, the same compressions a
sweep is made of) on one wave of chains per candidate, so a candidate costs about one boundary
family's worth of work per chain rather than a whole sweep.
"""
import time

import numpy as np

from . import _lib
from .engine import TnspError


def _sm_count(device):
    import torch
    return torch.cuda.get_device_properties(device).multi_processor_count


def tune_blocks_per_sm(sampler, configs, candidates=(1, 2, 3), device=0, repeats=1):
    """Times ``sampler.amplitude`` on one resident wave of configurations (cycled from ``configs``,
    shape (n, L1, L2)) for every blocks-per-SM candidate the kernel can hold, sets the fastest and
    returns (best, {candidate: amplitudes per second}).  Call after ``init_chains`` (the precision
    decides the kernel); it re-plans the per-block scratch, so call it before observing."""
    configs = np.asarray(configs, dtype=np.int32)
    sms = _sm_count(device)
    rates = {}
    for b in candidates:
        try:
            sampler.set_option(_lib.TNSP_OPT_BLOCKS_PER_SM, b)
            probe = configs[np.arange(b * sms) % len(configs)]
            sampler.amplitude(probe[:1])  # plans and allocates the slots
        except TnspError:
            continue  # more blocks than an SM can hold for this kernel and lattice
        best = None
        for _ in range(repeats):
            t0 = time.perf_counter()
            sampler.amplitude(probe)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        rates[b] = len(probe) / best
    if not rates:
        raise TnspError("no blocks-per-SM candidate fits this kernel")
    choice = max(rates, key=rates.get)
    sampler.set_option(_lib.TNSP_OPT_BLOCKS_PER_SM, choice)
    return choice, rates
