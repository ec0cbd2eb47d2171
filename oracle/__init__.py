"""CPU oracle for the EdelweissFE element-loop / VIJ->CSR / linear-solve hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg use it, and only as the checker (or the timed CPU baseline).

It is a plain numpy restatement of the reference algorithms, each function
citing the reference file:line it follows (paths relative to the EdelweissFE
source tree).  It is pinned against

* the reference's own golden solution files (``testfiles/*/U.ref``), copied
  into ``tests/golden/`` by ``tests/golden/make_golden.py``, and
* per-element / CSR / Newton-history fixtures produced by running the
  reference itself (same script).
"""
