"""Algorithmic work per binned pair -- the constants the benchmark's roofline
fractions use (one place, shared by bench.py and the docs).

FP32 flops per binned pair (separation and r_p^2: 3 sub + 2 mul + 1 add = 6;
weight product 1):
  wgg  F = 7
  wg+  F = 33  (+ raw dx', dy' 2; cos 2theta / sin 2theta from (dx'^2 - dy'^2)/q,
                2dx'dy'/q 8; two-component rotation 6; w e, (w e)^2 for e+ and
                ex 4; theta term ~4; tally 2)
  w++  F = 55  (+ second rotation 6, three products and their squares 12, less reuse)
Shared-memory atomic updates per binned pair (main fields M + jackknife fields
J per attribution; one attribution per pair on average in a periodic box):
  wgg  M = 3,  J = 3
  wg+  M = 9,  J = 6
  w++  M = 15, J = 9
"""

FLOPS_PER_PAIR = {0: 7, 1: 33, 2: 55}
SMEM_MAIN = {0: 3, 1: 9, 2: 15}
SMEM_JK = {0: 3, 1: 6, 2: 9}


def smem_updates_per_pair(which_corr: int, do_jk: bool, attributions: float = 1.0) -> float:
    return SMEM_MAIN[which_corr] + (attributions * SMEM_JK[which_corr] if do_jk else 0.0)
