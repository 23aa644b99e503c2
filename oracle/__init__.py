"""CPU oracle for the Orrery simulation hot path — TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.

A NumPy restatement of Orrery's engines (``src/lucivant_sim/engines.py``,
``src/lucivant_sim/simulator.py``, ``src/lucivant_sim/stabilizer.py``), each function citing the
reference lines it follows. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs
of ``bench.py`` may import it, and only as the reference results a test compares against or as
the timed CPU baseline. The product
(``lucivant_sim_gb300``) never imports it and has no CPU fallback.

Pinning: the oracle is checked against golden vectors generated by running Orrery 0.3.0 itself
(``tests/golden/make_golden.py``) and against Orrery's known-answer tests (the ⟨XX⟩ = 0.8 and
P(1) = e^-0.3 cases, reset and if/else counts, endianness), see ``tests/test_oracle_golden.py``.
"""
