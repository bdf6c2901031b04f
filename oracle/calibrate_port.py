"""Times the PyTorch-CPU port (``oracle/torch_port.py``) against the reference's
own AdaptiveMPS on the same CPU, for the 40-qubit Haar brickwork (depth 20,
chi_max 256, eps 1e-8, complex64).  Needs the reference source; not used at
test or bench time.

    python oracle/calibrate_port.py [/path/to/ATLAS-Q] [repeats]

Prints gates/s of both and the port/reference time ratio per repeat, and
checks that both end with the same bond dimensions.
"""
import os
import sys
import time
import types

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
REPEATS = int(sys.argv[2]) if len(sys.argv) > 2 else 2


def _stub_matplotlib():
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    plt = types.ModuleType("matplotlib.pyplot")
    plt.__getattr__ = lambda name: (lambda *a, **k: None)
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)


def main():
    _stub_matplotlib()
    sys.path.insert(0, os.path.join(REF, "src"))
    sys.path.insert(0, REPO)
    from atlas_q.adaptive_mps import AdaptiveMPS, DTypePolicy

    from atlasq_gb300.circuits import haar_brickwork
    from oracle.torch_port import TorchPortMPS

    torch.set_num_threads(os.cpu_count() or 1)
    ops = haar_brickwork(40, 20, seed=1234)
    for _ in range(REPEATS):
        t0 = time.perf_counter()
        ref = AdaptiveMPS(40, bond_dim=1, eps_bond=1e-8, chi_max_per_bond=256, device="cpu",
                          dtype=torch.complex64, dtype_policy=DTypePolicy(default=torch.complex64))
        for _, q, U in ops:
            ref.apply_two_site_gate(q, U)
        t_ref = time.perf_counter() - t0
        t0 = time.perf_counter()
        port = TorchPortMPS(40, eps_bond=1e-8, chi_max=256)
        for _, q, U in ops:
            port.apply_two_site_gate(q, U)
        t_port = time.perf_counter() - t0
        same = list(ref.bond_dims) == [t.shape[2] for t in port.tensors[:-1]]
        print(f"cores {os.cpu_count()}: reference {len(ops) / t_ref:.1f} gates/s, port {len(ops) / t_port:.1f} "
              f"gates/s, port/reference time {t_port / t_ref:.3f}, same bond dims {same}")


if __name__ == "__main__":
    main()
