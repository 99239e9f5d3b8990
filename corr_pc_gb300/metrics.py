"""Algorithmic work per binned pair -- the constants the benchmark's roofline
fractions use (one place, shared by bench.py and the docs).

FP32 flops per binned pair (separation and r_p^2: 3 sub + 2 mul + 1 add = 6;
weight product 1):
  wgg  F = 7
  wg+  F = 33  (+ raw dx', dy' 2; cos 2theta / sin 2theta from (dx'^2 - dy'^2)/q,
                2dx'dy'/q 8; two-component rotation 6; w e, (w e)^2 for e+ and
                ex 4; theta term ~4; tally 2)
  w++  F = 55  (+ second rotation 6, three products and their squares 12, less reuse)
  kappa-density (which_corr 3)  F = 8   (wgg + w kappa)
  shape-kappa   (which_corr 4)  F = 26  (wgg + angle 10, rotation 6, w kappa and
                                         its two products 3)
  ED            (which_corr 5)  F = 17  (wgg + dz^2 2, orientation dot product 5,
                                         its square over r^2 2, the square 1)
  r-mu binning (coordinates 7) adds 4: dz^2 into r^2, sqrt, mu = dz / r.
Shared-memory atomic updates per binned pair (main fields M + jackknife fields
J per attribution; one attribution per pair on average in a periodic box):
  wgg  M = 3,  J = 3
  wg+  M = 9,  J = 6
  w++  M = 15, J = 9
  kappa M = 4, J = 4;  shape-kappa M = 6, J = 6;  ED M = 5, J = 4
"""

FLOPS_PER_PAIR = {0: 7, 1: 33, 2: 55, 3: 8, 4: 26, 5: 17}
RMU_EXTRA_FLOPS = 4
SMEM_MAIN = {0: 3, 1: 9, 2: 15, 3: 4, 4: 6, 5: 5}
SMEM_JK = {0: 3, 1: 6, 2: 9, 3: 4, 4: 6, 5: 4}


def flops_per_pair(which_corr: int, coordinates: int = 6) -> int:
    return FLOPS_PER_PAIR[which_corr] + (RMU_EXTRA_FLOPS if coordinates == 7 else 0)


def smem_updates_per_pair(which_corr: int, do_jk: bool, attributions: float = 1.0) -> float:
    return SMEM_MAIN[which_corr] + (attributions * SMEM_JK[which_corr] if do_jk else 0.0)
