"""CPU oracle for the FBPINN training step — TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU, the algorithm of the reference library
(benmoseley/FBPINNs, ``fbpinns`` v0.2.0) for the path that the CUDA engine in
``fbpinns_gb300`` replaces.  It is the checker, never the thing that is
measured or shipped:

* only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
  ``--impl reference`` legs of ``bench.py`` may import it;
* nothing in ``fbpinns_gb300`` imports it, and the product path fails loudly
  when its CUDA library is missing instead of falling back to this code.

Modules
-------
``takes``   numpy restatement of the interaction-list construction
            (``fbpinns/decompositions_base.py:24-84``,
            ``fbpinns/decompositions.py:202-227``, ``fbpinns/trainers.py:332-419``,
            ``fbpinns/trainers.py:482-575``).  Integer work, compared bit-exactly.
``model``   torch (float64 by default) restatement of the model, the nested
            forward-mode derivative jets, the loss and its reverse-mode gradient
            (``fbpinns/trainers.py:63-267``), the decomposition / window / network
            / problem functions it calls, and optax's Adam.

Pinning
-------
The reference needs JAX, which is not installed, so it cannot be run as-is.
``tests/golden/make_golden.py`` runs the reference's own source files with
``jax.numpy`` replaced by numpy (float64) and writes golden vectors for the
interaction lists, decomposition parameters, per-pair model values, the POU
combination, constraining functions, losses and scheduler masks; the tests pin
this oracle against those vectors.  Derivative jets and parameter gradients
are pinned by float64 finite differences of the same golden forward values.
"""
