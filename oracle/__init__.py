"""Oracle: CPU restatement of the reference's table-mode NUFFT.

Test infrastructure only.  ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it as the
checker or the timed CPU baseline; the product package never imports it.
"""
