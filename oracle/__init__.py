"""CPU oracle for the scopyon image-formation path.

TEST INFRASTRUCTURE ONLY.  Nothing in ``scopyon_gb300`` imports this package.
It is imported by ``tests/``, by ``__graft_entry__.smoke()`` (as the checker of
one small GPU run) and by ``bench.py`` (the timed CPU baseline leg and
``--impl reference``).  It is an FP64 numpy restatement of the reference's
per-frame path, function by function, each citing the reference file:line it
follows (paths are relative to the ecell/scopyon source tree).

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against golden vectors produced by running the reference itself
(``tests/golden/make_golden.py``).
"""

from .epifm import *  # noqa: F401,F403
