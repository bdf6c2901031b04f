"""CPU oracle for the ATLAS-Q MPS hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory.  It is used by ``tests/``, by ``__graft_entry__.smoke()`` as the
checker, and by ``bench.py`` for the CPU baseline leg (``cpu_baseline`` and the
``--impl reference`` arm).  The GPU product path never routes through it.

The oracle is a NumPy restatement of the reference algorithm
(followthesapper/ATLAS-Q 0.7.0, ``src/atlas_q/adaptive_mps.py``,
``src/atlas_q/mps_pytorch.py``, ``src/atlas_q/truncation.py``,
``src/atlas_q/mpo_ops.py``, ``src/triton_kernels/mps_complex.py``); each
function cites the file:line it follows.  It is pinned against golden vectors
produced by running the reference itself (``tests/golden/make_golden.py``).

Modules:
    philox       -- Philox4x32-10 counter-based RNG (Salmon et al., SC'11).
    mps_oracle   -- AdaptiveMPS restatement (gates, truncation, canonical
                    sweeps, sampling, expectations, statistics).
    statevector  -- exact dense simulator using the reference's conventions.
    mlp_oracle   -- float64 forward/backward/Adam of the rank-predictor MLP.
"""
