"""Loads the golden vectors made by tests/golden/make_golden.py (reference outputs)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["heis_no_3x3_D3_dc4", "heis_no_4x4_D4_dc16", "heis_no_4x4_D3_dc5", "heis_u1_4x4_D111_dc5",
         "heis_u1_4x4_D222_dc8"]
# benchmark-size lattices (compact files: block storage, no holes, gradient on the allowed entries):
# 8x8 Bose U(1) D=6 with Dcut 36 (the throughput workload) and 6x6 Bose U(1) D=4 with Dcut 16
WORKLOAD_CASES = ["heis_u1_8x8_D222_dc36", "heis_u1_6x6_D121_dc16"]


class Golden:

    def __init__(self, name):
        self.name = name
        self.z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        self.meta = json.loads(str(self.z["meta"]))
        self.L1 = self.meta["L1"]
        self.L2 = self.meta["L2"]
        self.cut = self.meta["cut"]

    def dense_sites(self):
        if not self.meta.get("compact"):
            return [[self.z[f"site_{l1}_{l2}_dense"] for l2 in range(self.L2)] for l1 in range(self.L1)]
        from tnsp_gb300.lattice import site_from_blocks
        out = []
        for l1 in range(self.L1):
            row = []
            for l2 in range(self.L2):
                meta = self.meta["sites"][f"{l1},{l2}"]
                row.append(site_from_blocks(self.z[f"site_{l1}_{l2}_storage"], [m["name"] for m in meta],
                                            [[tuple(x) for x in m["segments"]] for m in meta]))
            out.append(row)
        return out

    def gradient(self, l1, l2, dense=None):
        """The reference's gradient of site (l1, l2) as a dense (P0, U, D, L, R) array."""
        if not self.meta.get("compact"):
            return self.z[f"grad_{l1}_{l2}"]
        site = (dense or self.dense_sites())[l1][l2]
        g = np.zeros_like(site)
        g[site != 0] = self.z[f"grad_{l1}_{l2}_allowed"]
        return g

    def terms(self):
        """[(positions, {s_in: [(s_out, value), ...]})] in the reference's dictionary order."""
        out = []
        for ti, t in enumerate(self.meta["terms"]):
            pos = tuple(tuple(p) for p in t["positions"])
            body = len(pos)
            table = {}
            for r in self.z[f"term_{ti}_table"]:
                si = tuple(int(x) for x in r[:body])
                so = tuple(int(x) for x in r[body:2 * body])
                table.setdefault(si, []).append((so, float(r[-1])))
            out.append((pos, table))
        return out

    def neel(self):
        return np.fromfunction(lambda a, b: (a + b) % 2, (self.L1, self.L2)).astype(np.int64)
