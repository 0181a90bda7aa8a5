"""CPU oracle for the Qaintensor.jl hot path (test infrastructure only).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  It restates, in numpy/scipy FP64
(complex128) with Julia's column-major index order, the reference algorithms
that the CUDA engine replaces:

* ``contract_rep`` / ``ncon`` pairwise contraction   (src/contract.jl:39-60, 242-264)
* ``contract_order`` contraction-order search        (src/contract.jl:8-32, 65-235)
* ``contract_svd`` and its absolute tail-norm rule    (src/svd.jl:7-38, rule at :29-33)
* ``switch!`` / ``permute!``                          (src/switch.jl:6-106)
* ``MPS(psi)`` sequential SVD                         (src/mps.jl:55-89)
* ``MPO(m)`` / ``decompose!``                         (src/mpo.jl:27-90, src/decompose.jl:6-52)
* ``extend_MPO`` / ``apply_MPO`` wiring               (src/mpo.jl:122-252)
* ``tensor_circuit!`` lazy gate insertion             (src/tensor_circuit.jl:14-80)

plus the documented extensions the engine adds on top of those conventions:
the composed two-qubit gate + truncated-SVD update, Haar gates, brickwork
circuits, expectation values, the transverse-field Ising MPO and the SVD
compression sweep, and the FP64 rank-predictor MLP.

The reference is pure Julia and cannot run in this image (no Julia); the
oracle is pinned by porting the reference's own equivalence tests
(test/test_svd.jl, test/test_mps.jl, test/test_mpo.jl,
test/test_tensor_circuit.jl) to ``tests/test_oracle_*.py``.
"""

from .reference_path import *  # noqa: F401,F403
from .extensions import *  # noqa: F401,F403
