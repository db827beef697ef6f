"""Timed CPU baseline of one amplitude update (TEST INFRASTRUCTURE ONLY).

Used by ``bench.py`` for its ``cpu_baseline`` object and for the
``--impl reference`` arm: the reference itself (spin-orbital arrays) cannot
hold the o=24/v=300 system, so the timed CPU implementation is this
repository's FP64 closed-shell restatement (``oracle.ccsd_rhf``), run by
numpy on all host cores, on a bounded sample of one update:

* every residual term except the particle-particle ladder is computed in full;
* the ladder sum_cd (ac|bd) tau_ij^cd is computed for ``ladder_rows`` of the
  v virtual rows a (with the (ac|bd) rows built from the DF factors inside the
  timed region) and scaled by v / ladder_rows;
* the integral blocks (o/v-blocks from the DF factors) are built once,
  outside the timed region, as the GPU engine builds them in ccsd_create.
"""
from __future__ import annotations

import os
import time

import numpy as np

from .ccsd_rhf import RHFCCSD


class SampledUpdate:
    def __init__(self, fock: np.ndarray, nocc: int, df: np.ndarray, ladder_rows: int = 3):
        self.cc = RHFCCSD(fock, nocc, df=df, with_vvvv=False)
        self.cc.skip_ladder = True
        self.rows = max(1, min(ladder_rows, self.cc.v))
        self.t1, self.t2 = self.cc.mp2_guess()

    def step(self) -> dict:
        """Time one sampled update; returns the extrapolated seconds."""
        cc = self.cc
        t0 = time.perf_counter()
        R1, R2 = cc.residual(self.t1, self.t2)
        t1 = time.perf_counter()
        tau = cc.tau(self.t1, self.t2)
        part = cc.ladder_rows(tau, 0, self.rows)
        t2 = time.perf_counter()
        R2[:, :, :self.rows, :] += part
        scale = cc.v / self.rows
        return dict(seconds=(t1 - t0) + (t2 - t1) * scale, rest_s=t1 - t0,
                    ladder_sample_s=t2 - t1, ladder_scale=scale)


def cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
