"""TEST ORACLE -- CPU restatements of jax-powspec's P(k) path.

This package is test infrastructure, not product code.  Only tests/,
__graft_entry__.smoke() and the CPU-baseline leg of bench.py may import it,
and only as the checker (or as the timed CPU stand-in for the reference).

  reference_f32   numpy float32 restatement of src/mas.py and the P(k) part
                  of src/correlations.py, reference bugs included
  truth_f64       FP64 estimator of the same P_l(k) the GPU computes
                  (all mass-assignment orders, interlacing, shot noise)
"""
