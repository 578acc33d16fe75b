"""CPU oracle for the marginal-likelihood / rejection hot path.

Test infrastructure only: tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may use it.  The product package
``thejoker_gb300`` never imports anything from here.
"""
