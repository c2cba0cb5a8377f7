"""CPU oracle for the geepee sparse-GP layer path.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` (as the
checker) and ``bench.py``'s CPU-baseline / reference arm.  The product package
``geepee_gb300`` never imports it, and nothing here is shipped or measured as the
GPU path.

* ``oracle.geepee_np`` - float64 numpy restatement of the reference algorithm
  (thangbui/geepee ``geepee/kernels.py``, ``base_models.py``, ``aep_models.py``,
  ``lik_layers.py``, ``utils.py``), each function citing the lines it follows.
* ``oracle/psi_c.c``   - plain C restatement of the psi-statistics loop
  (``geepee/kernels.py:201-234``), used as the timed scalar CPU baseline.
* ``oracle/make_ref.py`` - recipe that builds ``oracle/_ref/`` (git-ignored) from
  the reference sources: a Python 3 shim of the reference package and the
  reference's own weave C++ loop as a compilable file.

Parity pin: ``tests/golden/*.npz`` were generated by ``tests/golden/make_golden.py``
from the reference's own code (through ``oracle/_ref``) and
``tests/test_oracle_golden.py`` checks this oracle against them.
"""
