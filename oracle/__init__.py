"""CPU oracle for the MUSCL + HLL + hydrostatic SSP-RK3 hot path.

TEST INFRASTRUCTURE ONLY.  ``oracle.port`` binds the C restatement
(``oracle/swe_oracle.c``, built on every machine by ``oracle/Makefile``);
``oracle.ref`` binds the reference's own solver compiled from its sources
(``oracle/_ref``, present only where the reference sources are).  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this package; the shipped library never does.
"""
