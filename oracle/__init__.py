"""CPU oracle of the reference fitter.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the product package.

* ``OracleModel`` - the C++ restatement (lm_oracle.hpp) compiled for one
  generated model; float/float, float/double and double/double modes.
* ``RefIVIM`` - the reference's own generated IVIM kernel built as host C++
  (oracle/_ref, see the Makefile), for 21 or 10 b-values. Only present where
  the reference tree was available at build time.
"""
from .build import OracleModel, RefIVIM, build_reference, ref_available  # noqa: F401
