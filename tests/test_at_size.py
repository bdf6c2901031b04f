"""The secondary workloads at their stated sizes against the FP64 oracle.

* 50 qubits, Haar brickwork depth 16, chi_max 256 (complex64), the sampling
  and expectation workload: 4096 shots decision by decision against the
  oracle's sampler (right-canonical form in float64, the same Philox4x32-10
  uniforms): every shot agrees, or its first differing decision lies within
  1e-4 of the oracle's P(0) (float32 probabilities at 50 sites); and all 49
  <Z_i Z_i+1> plus 50 <X_i> within 1e-6 of the oracle evaluated in float64 on
  the same tensors, computed from the complex128 copy of the state (the
  complex64 evaluation is checked at 1e-5).
* 64-qubit hardware-efficient ansatz, chi_max 512: three layers against the
  oracle's complex128 run: the kept rank of every gate (either precision's
  choice where a float32 threshold sits on a degenerate pair) and fidelity
  > 1 - 1e-6.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import atlasq_gb300 as aq  # noqa: E402
from atlasq_gb300.circuits import haar_brickwork, hea_circuit  # noqa: E402
from atlasq_gb300.sampling import right_canonical_copy, sample_tensors  # noqa: E402
from oracle import mps_oracle as mo  # noqa: E402
from oracle.philox import sample_uniforms  # noqa: E402

DEV = "cuda:0"


@pytest.fixture(scope="module")
def state50():
    m = aq.AdaptiveMPS(50, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=256, device=DEV, device_resident=True)
    for _, q, U in haar_brickwork(50, 16, seed=77):
        m.apply_two_site_gate(q, U)
    m.flush()
    assert max(m.bond_dims) == 256
    return m


def test_sampling_50q_chi256_decision_exact(state50):
    shots, seed = 4096, 5
    ts = right_canonical_copy(state50)
    bits, pz = sample_tensors(ts, shots, seed, return_pz=True)
    bits = bits.cpu().numpy()
    rc = mo.right_canonicalize([t.cpu().numpy() for t in state50.tensors])
    ref_bits, ref_pz = mo.batch_sweep_sample(rc, shots, seed)
    n = 50
    diff = np.nonzero(bits != ref_bits)[0]
    for s in diff:
        x = int(bits[s]) ^ int(ref_bits[s])
        site = n - x.bit_length()  # first differing decision (qubit 0 is the MSB)
        u = sample_uniforms(seed, np.array([s], dtype=np.uint64), site)[0]
        assert abs(u - ref_pz[s, site]) < 1e-4, (s, site, u, ref_pz[s, site])
    assert len(diff) <= shots // 100, len(diff)
    # the decisions before the first flip used the same probabilities
    same = bits == ref_bits
    assert np.max(np.abs(pz.cpu().numpy()[same] - ref_pz[same])) < 1e-4


def test_expectations_50q_chi256_vs_fp64(state50):
    X = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex64)
    Z = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex64)
    obs = [{i: Z, i + 1: Z} for i in range(49)] + [{i: X} for i in range(50)]
    host = [t.cpu().numpy() for t in state50.tensors]
    ref = np.array(mo.local_expectations(host, [{k: v.numpy() for k, v in o.items()} for o in obs]))
    got64 = np.array(aq.local_expectations(state50, obs))
    assert np.max(np.abs(got64 - ref)) < 1e-5, np.max(np.abs(got64 - ref))
    c128 = torch.complex128
    m2 = aq.AdaptiveMPS(50, bond_dim=1, device=DEV, dtype=c128, dtype_policy=aq.DTypePolicy(default=c128))
    m2.tensors = [t.to(c128) for t in state50.tensors]
    m2.bond_dims = list(state50.bond_dims)
    got128 = np.array(aq.local_expectations(m2, [{k: v.to(c128) for k, v in o.items()} for o in obs]))
    assert np.max(np.abs(got128 - ref)) < 1e-6, np.max(np.abs(got128 - ref))


def test_hea64_chi512_three_layers_vs_oracle():
    ops_ = hea_circuit(64, 3, seed=64)
    m = aq.AdaptiveMPS(64, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=512, device=DEV)
    o64 = mo.OracleMPS(64, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=512, dtype=np.complex64)
    o128 = mo.OracleMPS(64, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=512, dtype=np.complex128)
    for kind, q, U in ops_:
        if kind == "2q":
            m.apply_two_site_gate(q, U)
            o64.apply_two_site_gate(q, U.numpy())
            o128.apply_two_site_gate(q, U.numpy())
        else:
            m.apply_single_qubit_gate(q, U)
            o64.apply_single_qubit_gate(q, U.numpy())
            o128.apply_single_qubit_gate(q, U.numpy())
    m.flush()
    ks = m.statistics.logs["k_star"]
    k64, k128 = o64.logs["k_star"], o128.logs["k_star"]
    assert len(ks) == len(k128) == 3 * 63
    assert all(k in (a, b) for k, a, b in zip(ks, k64, k128)), [(k, a, b) for k, a, b in zip(ks, k64, k128)
                                                                if k not in (a, b)]
    f = mo.mps_fidelity([t.cpu().numpy() for t in m.tensors], o128.tensors)
    assert f > 1 - 1e-6, f
