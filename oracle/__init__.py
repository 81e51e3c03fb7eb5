"""ORACLE -- test infrastructure, never product code.

ctypes bindings to the CPU checkers built by oracle/Makefile:

* ``liboracle.so``       the C restatement of gala's hot path (gx_oracle.c,
                         scf_oracle.c), strict IEEE order: the parity checker;
* ``liboracle_fast.so``  the same source with gala's own flags (-Ofast): the
                         CPU baseline timed by bench.py;
* ``libgalaref.so``      gala's own C/C++ compiled from the gala sources (only
                         where those sources are present), used to pin the
                         restatement and to generate tests/golden fixtures.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package.
"""
from .oracle import Oracle, build, ref_available  # noqa: F401
