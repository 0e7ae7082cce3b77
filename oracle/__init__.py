"""FP64 NumPy oracle for the SPI-Active batched candidate-evaluation path.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports this
package. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may use it, and only as the checker or as the timed CPU
baseline, never as the thing measured on the GPU.

What it restates, and against what it is pinned:

* Formula-level pieces of the reference (PD law, action clip, motor models,
  window construction, reference cost and normaliser, FD-Fisher proxy,
  command parametrisations). These are pinned by golden vectors that
  ``tests/golden/make_golden.py`` produced by executing the reference's own
  functions (extracted from its source files) on seeded inputs.
* The rigid-body dynamics (floating-base ABA, penalty ground contact,
  semi-implicit Euler). The reference delegates them to Isaac Gym / PhysX, a
  closed binary that is not installable here, so **dynamics parity with the
  reference is unpinned**. The oracle's dynamics are instead validated by
  internal invariants (inverse-dynamics round trip through RNEA, CRBA mass
  matrix symmetry / positive definiteness, momentum conservation in free
  flight, free fall, quaternion norm).
"""
