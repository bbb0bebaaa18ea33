"""CPU checkers for the MIC step (test infrastructure only).

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, and nowhere else: the product package never imports this.

* ``Restatement`` -- ctypes front-end of oracle/v2c_oracle.c, the FP64 C
  restatement of the reference routines over explicit arrays.
* ``run_reference`` -- runs the reference's own routines (compiled from its
  sources by oracle/build_ref.sh into oracle/_ref/v2c_ref) on a case.
"""
from .bindings import (Restatement, build, reference_available,
                       restatement_path, run_reference, reference_path)

__all__ = ["Restatement", "build", "reference_available", "restatement_path",
           "run_reference", "reference_path"]
