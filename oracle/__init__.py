"""CPU oracle for the VEGAS+ loop of emiliantolo/cuvegas.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
package, and only as the checker or the timed CPU baseline.  The product
(``cuvegas_gb300``) never imports it.
"""
