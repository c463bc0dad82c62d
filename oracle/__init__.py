"""CPU oracle for the MPDO noisy-circuit hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only
as the checker or as the timed CPU baseline.

* :mod:`oracle.mpdo_oracle` restates the reference's MPDO path (gate and Kraus
  contraction, the 2-site SVD split, the QR left-to-right and SVD
  right-to-left truncation sweeps, the kappa-truncating SVD and the
  density-matrix readout) in plain torch on the CPU.
* :mod:`oracle.dense_dm` is an exact dense density-matrix simulator (n <= 10)
  used as a physics pin.

Parity pin: the restatement is checked against outputs of the reference's own
code run in this container (``tests/golden/make_golden.py``, which imports the
reference with a stand-in for its absent TensorNetwork dependency) and against
the dense simulator.
"""
