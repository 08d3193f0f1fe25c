"""The sampler kernel's fermionic integer logic, compiled for the host from
tnsp_gb300/csrc/sampler_kernels.cuh, against the oracle, which the reference's own outputs pin
(tests/test_fermi_peps.py): the E_loc term sign (``fermion_term_sign`` / ``config_sign_bit``: the hop
string and, for a vertical pair, the column / row configuration signs and the order inversions), the
prefix counts that pick a site's slice (``strip_prefix_of``, and the rule by which a replaced pair's
second site counts the first one's new occupation), and the slice index (``fermion_slice``)."""
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
  int mode;
  short conf[256];
  while (scanf("%d", &mode) == 1) {
    if (mode == 0) {  // E_loc term sign
      int L1, L2, pT, ia, na, ib, nb, vertical;
      scanf("%d %d %d %d %d %d %d %d", &L1, &L2, &pT, &ia, &na, &ib, &nb, &vertical);
      for (int i = 0; i < L1 * L2; ++i) { int v; scanf("%d", &v); conf[i] = (short)v; }
      printf("%d\n", (int)tnsp::fermion_term_sign(conf, L1, L2, pT, ia, na, ib, nb, vertical));
    } else if (mode == 1) {  // strip prefix
      int L1, L2, kind, idx, c;
      scanf("%d %d %d %d %d", &L1, &L2, &kind, &idx, &c);
      for (int i = 0; i < L1 * L2; ++i) { int v; scanf("%d", &v); conf[i] = (short)v; }
      printf("%d\n", tnsp::strip_prefix_of(conf, L2, kind, idx, c));
    } else {  // slice index
      int orient, s, mp;
      scanf("%d %d %d", &orient, &s, &mp);
      printf("%lld\n", tnsp::fermion_slice(orient, s, mp));
    }
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
        lines.append(f"0 {L1} {L2} {pT} {ia} {new[0]} {ib} {new[1]} {vertical} " + " ".join(map(str, conf.ravel())))
    out = subprocess.run([harness], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    got = [int(x) for x in out.stdout.split()]
    assert got == want


def test_kernel_prefix_and_slice_equal_the_host_tables(harness):
    from tnsp_gb300 import fermion as F
    rng = np.random.default_rng(29)
    lines, want = [], []
    for _ in range(300):
        L1, L2 = int(rng.integers(2, 7)), int(rng.integers(2, 7))
        conf = (rng.random((L1, L2)) < 0.5).astype(np.int64)
        kind = int(rng.integers(0, 2))
        idx = int(rng.integers(0, L1 if kind == 0 else L2))
        c = int(rng.integers(0, L2 if kind == 0 else L1))
        l1, l2 = (idx, c) if kind == 0 else (c, idx)
        want.append(int(fp.prefix_counts(conf, fp.ROW if kind == 0 else fp.COL)[l1, l2]))
        lines.append(f"1 {L1} {L2} {kind} {idx} {c} " + " ".join(map(str, conf.ravel())))
    layout = np.arange(8).reshape(2, 2, 2)   # sign_folded_slices: [family][n][prefix parity]
    for orient in range(4):
        for s in (0, 1):
            for mp in range(4):
                want.append(int(layout[1 if orient >= 2 else 0, s, mp & 1]))
                lines.append(f"2 {orient} {s} {mp}")
    out = subprocess.run([harness], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    assert [int(x) for x in out.stdout.split()] == want
    # a replaced pair: the second site's prefix is the first site's prefix plus the first site's new value
    for _ in range(200):
        L1, L2 = int(rng.integers(2, 6)), int(rng.integers(2, 6))
        conf = (rng.random((L1, L2)) < 0.5).astype(np.int64)
        vertical = bool(rng.integers(0, 2))
        a, b = (int(rng.integers(0, L1 - 1)), int(rng.integers(0, L2))) if vertical else \
            (int(rng.integers(0, L1)), int(rng.integers(0, L2 - 1)))
        p0, p1 = (a, b), ((a + 1, b) if vertical else (a, b + 1))
        s0, s1 = int(rng.integers(0, 2)), int(rng.integers(0, 2))
        after = conf.copy()
        after[p0], after[p1] = s0, s1
        fam = F.COL if vertical else F.ROW
        M, Ma = fp.prefix_counts(conf, fam), fp.prefix_counts(after, fam)
        assert Ma[p0] == M[p0] and Ma[p1] == M[p0] + s0
