"""Generate the sampler fixtures of tests/golden/ by running the reference's network.

Run in a container that holds the reference source tree (qmb-public):

    python tests/golden/make_sampler_golden.py --reference /path/to/qmb-public

It imports the reference's ``qmb.mlp.WaveFunctionElectronUpDown`` (plain
PyTorch, CPU), builds it with a seeded initialisation, evaluates its
``forward`` on seeded configurations and runs ``generate_unique`` while
recording every uniform tensor its Gumbel perturbation draws
(``torch.rand_like``), and writes one ``.npz`` per case: the network's
parameters (state_dict entries), the inputs, the recorded uniforms and the
reference's outputs.  The tests read only the fixtures.
"""

from __future__ import annotations

import argparse
import pathlib
import sys

import numpy as np
import torch

HERE = pathlib.Path(__file__).resolve().parent

CASES = {
    # name: (sites, spin_up, spin_down, hidden, ordering, batch, seed)
    "sampler_6": (6, 3, 3, (16, 16), +1, 60, 11),
    "sampler_14": (14, 5, 5, (64,), -1, 3000, 12),
    "sampler_10_custom": (10, 4, 3, (32, 32), [3, 1, 4, 0, 9, 2, 6, 5, 8, 7], 500, 13),
}


def main() -> None:
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", required=True)
    args = parser.parse_args()
    sys.dont_write_bytecode = True
    sys.path.insert(0, args.reference)
    import qmb.bitspack  # type: ignore
    import qmb.mlp  # type: ignore

    for name, (sites, up, down, hidden, ordering, batch, seed) in CASES.items():
        torch.manual_seed(seed)
        net = qmb.mlp.WaveFunctionElectronUpDown(double_sites=2 * sites, physical_dim=2, is_complex=True,
                                                 spin_up=up, spin_down=down, hidden_size=hidden, ordering=ordering)
        # larger weights than the default initialisation, so that the sampled
        # distribution is far from uniform
        with torch.no_grad():
            for p in net.parameters():
                p.mul_(3.0)
        state = {k: v.detach().numpy().copy() for k, v in net.state_dict().items()}
        # forward on random valid configurations
        gen = np.random.default_rng(seed)
        rows = []
        for _ in range(64):
            bits = np.zeros((sites, 2), dtype=np.uint8)
            bits[gen.choice(sites, up, replace=False), 0] = 1
            bits[gen.choice(sites, down, replace=False), 1] = 1
            rows.append(bits.reshape(-1))
        configs = qmb.bitspack.pack_int(torch.from_numpy(np.stack(rows)), size=1)
        with torch.no_grad():
            psi = net(configs)
        # generate_unique with the Gumbel uniforms recorded
        recorded = []
        original = torch.rand_like

        def recording(t, *a, **k):
            u = original(t, *a, **k)
            recorded.append(u.detach().numpy().copy())
            return u

        torch.rand_like = recording
        try:
            with torch.no_grad():
                x, amp, _, _ = net.generate_unique(batch)
        finally:
            torch.rand_like = original
        out = {f"param:{k}": v for k, v in state.items()}
        out.update({f"uniform:{i}": u for i, u in enumerate(recorded)})
        out.update(configs=configs.numpy(), psi=psi.numpy(), sampled=x.numpy(), sampled_psi=amp.numpy(),
                   sites=np.int64(sites), spin_up=np.int64(up), spin_down=np.int64(down),
                   hidden=np.array(hidden, dtype=np.int64), ordering=np.array(net.ordering.numpy(), dtype=np.int64),
                   batch=np.int64(batch))
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, "sampled", x.shape[0], "rows; uniforms", len(recorded))


if __name__ == "__main__":
    main()
