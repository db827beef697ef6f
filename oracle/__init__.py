"""CPU oracle for the CCSD amplitude iteration (TEST INFRASTRUCTURE ONLY).

Nothing in the product path imports this package.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may use it, and only as the reference the GPU results are
compared with or as the timed CPU baseline -- never as the thing that is
measured or shipped.

Contents
--------
``synthetic``      seeded generator for the density-fitted synthetic systems
                   (orbital energies + B^Q_pq factors), counter-based so that
                   the C++ generator in the library reproduces it.
``ccsd_spinorb``   FP64 spin-orbital CCSD, a restatement of the reference's
                   dense CCSD equations (``ccsdt.cpp`` with ``Method_Nr == -1``)
                   driven with the iteration semantics of
                   ``CCSD_Memory_optimized::CCSD`` (``ccsd_memory_optimized.cpp``).
``ccsd_rhf``       FP64 closed-shell (spin-adapted) restatement of the same
                   iteration map, for the shapes where spin orbitals do not
                   fit; checked against ``ccsd_spinorb`` at small sizes.
``ref_build/``     recipe that compiles the reference's own C++ sources
                   (unchanged) against a small Armadillo-subset shim and a
                   single-rank MPI stub into ``oracle/_ref/``; its outputs pin
                   the restatements.
"""
