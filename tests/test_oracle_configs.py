"""The CPU oracle against the digests recorded from the reference's own CPU
library at the measured configurations' sizes: the 32x32 Izhikevich network
for all 1000 steps, and the three-layer 256x256 plastic network for its first
10 steps (the GPU tests run it for all 1000)."""
import numpy as np

from tests.golden import configs
from tests.harness import load_fixture, run_oracle_digest


def _same(got, want, steps):
    for k, g in got.items():
        if k.startswith("digest/") or k.startswith("count/"):
            bad = np.flatnonzero(g != want[k][:steps])
            assert bad.size == 0, "%s differs from step %d" % (k, bad[0])
        elif k.startswith("final@"):
            assert g[0] == want[k][0], k


def test_oracle_c0_1000_steps():
    case = configs.c0_case()
    _same(run_oracle_digest(case, 1000, configs.CHECKPOINTS), load_fixture(case.name), 1000)


def test_oracle_c2_first_steps():
    case = configs.c2_case()
    got = run_oracle_digest(case, 10)
    _same({k: v for k, v in got.items() if not k.startswith("final@")}, load_fixture(case.name), 10)
