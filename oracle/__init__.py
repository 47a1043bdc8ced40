"""CPU oracle for libtnfa -- TEST INFRASTRUCTURE ONLY.

A plain numpy restatement of ITensorNumericalAnalysis.jl's algorithms
(digit maps, constructors, direct sum / Hadamard product, OpSum operators
applied exactly on the dense grid, evaluation, integration, bond spectra),
written with labelled tensors the way ITensors.jl writes them.  Each
function cites the reference file:line it restates.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package, and only to check or time; the product
(itensornumericalanalysis) never imports it.

Pinning: the reference (Julia, ITensorNetworks 0.13) cannot run in this
environment, so the oracle is pinned against the reference's own known-answer
tests (test/test_indexmaps.jl, test/test_realitensorfunction.jl,
test/test_complexitensorfunction.jl, test/test_operators.jl,
test/test_integration.jl), restated in tests/test_oracle_pins.py.
"""
from .itn import *  # noqa: F401,F403
