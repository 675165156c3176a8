"""CPU checkers for the photon trace (test infrastructure only).

``bindings.Oracle`` wraps the C++ restatement built from this directory;
``bindings.Reference`` wraps the reference MARX library compiled in place
from its own sources (only where those sources are present).  Only the
tests, ``__graft_entry__.smoke`` and the bench's CPU-baseline leg use them.
"""
