"""CPU oracle for the Delta2 contact hot path (test infrastructure only).

A plain-C++ restatement of the reference's narrow phase, continuous
collision detection, time-step selection, sequential-impulse solve and
adaptive cluster stepper.  Loaded by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``; the product never imports it.
"""
