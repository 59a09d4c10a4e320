"""CPU oracle for the caustica k-space CW solver and its Pennes/CEM43 step.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports this
package. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may call it, and only as the checker (or, in
``bench.py --impl reference``, as the timed stand-in for the reference's own
NumPy CPU path, which is pure Python and cannot be shipped to the GPU host).

The modules restate, in plain NumPy/SciPy, the algorithm of the reference
(ebx0/caustica, Python) for this one path, citing the reference file:line
each function follows (paths relative to ``src/caustica/``):

* :mod:`oracle.kspace`  -- ``solvers/kspace/engine.py``, ``operators.py``,
  ``core/pml.py``, ``sources.py`` (ramp), ``solvers/base.py`` (interior).
* :mod:`oracle.pennes`  -- ``thermal/pennes.py``, ``thermal/dose.py``.
* :mod:`oracle.sensors` -- ``sensors.py`` (Q from phasors).

Both run in a chosen dtype. ``float64`` reproduces the reference engine run
through an FP64 backend (every ``xp.float32`` read as float64), which is the
parity oracle; ``float32`` reproduces the reference's stock NumPy path, which
is the CPU baseline. Parity pin: ``tests/golden/make_golden.py`` runs the
unchanged reference in FP64 on small cases and commits inputs and outputs;
``tests/test_oracle_golden.py`` holds this restatement to them.
"""
