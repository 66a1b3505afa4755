"""CPU oracle of the ray-tracing hot path — TEST INFRASTRUCTURE ONLY.

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU legs (the
cpu_baseline leg and ``--impl reference``).  The product library never links
or calls anything here.
"""
