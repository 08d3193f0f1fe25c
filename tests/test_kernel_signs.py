"""The sampler kernel's fermionic E_loc sign (``fermion_term_sign`` / ``config_sign_bit`` in
tnsp_gb300/csrc/sampler_kernels.cuh, compiled for the host here) against the oracle's, which the
reference's own local energies pin (tests/test_fermi_peps.py): the hop string and, for a vertical pair,
the column / row configuration signs and the order inversions."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import fermi_peps as fp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = r'''
#include <cstdio>
#include "sampler_kernels.cuh"
int main() {
  int L1, L2, pT, ia, na, ib, nb, vertical;
  short conf[256];
  while (scanf("%d %d %d %d %d %d %d %d", &L1, &L2, &pT, &ia, &na, &ib, &nb, &vertical) == 8) {
    for (int i = 0; i < L1 * L2; ++i) { int v; scanf("%d", &v); conf[i] = (short)v; }
    printf("%d\n", (int)tnsp::fermion_term_sign(conf, L1, L2, pT, ia, na, ib, nb, vertical));
  }
  return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("signs")
    src = d / "harness.cu"
    src.write_text(HARNESS)
    exe = d / "harness"
    subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(ROOT, "tnsp_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    return str(exe)


def test_kernel_term_sign_equals_the_oracle(harness):
    rng = np.random.default_rng(23)
    lines, want = [], []
    for _ in range(600):
        L1, L2 = int(rng.integers(2, 7)), int(rng.integers(2, 7))
        conf = (rng.random((L1, L2)) < 0.5).astype(np.int64)
        pT = int(rng.integers(0, 2))
        vertical = int(rng.integers(0, 2))
        if vertical:
            a, b = int(rng.integers(0, L1 - 1)), int(rng.integers(0, L2))
            p0, p1 = (a, b), (a + 1, b)
        else:
            a, b = int(rng.integers(0, L1)), int(rng.integers(0, L2 - 1))
            p0, p1 = (a, b), (a, b + 1)
        if conf[p0] == conf[p1]:
            conf[p1] = 1 - conf[p0]
        new = [int(conf[p1]), int(conf[p0])]  # the particle hops
        after = conf.copy()
        after[p0], after[p1] = new
        s = fp.hop_sign(conf, [p0, p1], new)
        if vertical:
            s *= fp.configuration_sign(after, pT, fp.COL) * fp.configuration_sign(conf, pT, fp.ROW) * \
                (-1.0)**fp.order_inversions(after)
        want.append(int(s))
        ia, ib = p0[0] * L2 + p0[1], p1[0] * L2 + p1[1]
        lines.append(f"{L1} {L2} {pT} {ia} {new[0]} {ib} {new[1]} {vertical} " + " ".join(map(str, conf.ravel())))
    out = subprocess.run([harness], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    got = [int(x) for x in out.stdout.split()]
    assert got == want
