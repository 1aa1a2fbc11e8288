"""CPU oracle for the closed-shell CCSD(T) hot path of sisi4s.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, the C++
host runner, the ``sisi4s_gb300`` package) imports, links or executes this
package.  It is used by ``tests/`` as the checker, by
``__graft_entry__.smoke()`` as the checker, and by ``bench.py`` only for its
``cpu_baseline`` leg and for ``--impl reference``.

What it is: a numpy restatement of the reference's CTF statements, one
``einsum`` per statement and in the same order, for

* ``CoulombIntegralsFromVertex`` real integrals
  (src/algorithms/CoulombIntegralsFromVertex.cxx:203-558)    -> ``coulomb.py``
* ``CcsdEnergyFromCoulombIntegrals::getResiduum`` real path
  (src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:27-494) -> ``ccsd.py``
* ``CcsdEnergyFromCoulombIntegralsReference::getResiduum``
  (src/algorithms/CcsdEnergyFromCoulombIntegralsReference.cxx:29-295),
  the stored-Vabcd formulation used as an independent cross-check -> ``ccsd.py``
* ``ClusterSinglesDoublesAlgorithm`` driver, Jacobi update, energy
  (src/algorithms/ClusterSinglesDoublesAlgorithm.cxx:38-364,888-915) -> ``ccsd.py``
* ``DiisMixer`` / ``LinearMixer`` (src/mixers/DiisMixer.cxx:16-180,
  src/mixers/LinearMixer.cxx:30-44)                             -> ``mixers.py``
* ``CcsdPerturbativeTriples`` (src/algorithms/CcsdPerturbativeTriples.cxx:32-248,
  src/math/Permutation.hpp:50-118)                              -> ``triples.py``
* ``UegVertexGenerator`` (src/algorithms/UegVertexGenerator.cxx:10-229) -> ``ueg.py``
* the complex (k-point) branch: complex integrals
  (src/algorithms/CoulombIntegralsFromVertex.cxx:613-816), the complex
  residual (src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:496-891), the
  complex driver with the linear mixer, and ``CcsdPerturbativeTriplesComplex``
  (src/algorithms/CcsdPerturbativeTriplesComplex.cxx:32-348) -> ``ccsd_complex.py``

Parity pin: the reference itself cannot be built here (Cyclops CTF, MPI and
yaml-cpp are absent), so the oracle is pinned against the golden energies of
the reference's own integration test ``tests/cc4s/ueg/rs1.0-7occ-26virt``
(``cc4s.correct.out.yaml:120-169``: MP2, CCSD and (T) energies).  That test's
input vertex is downloaded at test time; ``ueg.py`` regenerates the same
system from the restated ``UegVertexGenerator`` and rotates it to a real
(standing-wave) orbital basis, which the reference's real code path assumes.
The oracle reproduces those three golden numbers (see
``tests/test_oracle_pin.py``).  The complex branch reproduces them too, on
the plane-wave vertex itself made complex by random orbital phases (see
``tests/test_oracle_complex.py``).
"""
