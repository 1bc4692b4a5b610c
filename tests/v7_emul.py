"""Pure-Python port of the reference's v7 block executor (batch_engine_v7.hpp:832-968)
over the gpu_v7_launch argument arrays: phase 1 per-block local Fenwick replay with
row and factor nodes, phase 2 serial carry, phase 3 combine.  Test infrastructure,
small cases only."""
from __future__ import annotations

import numpy as np

MASK = (1 << 64) - 1


def s64(x: int) -> int:
    x &= MASK
    return x - (1 << 64) if x >> 63 else x


def run(plan: dict):
    B, G, Cp, ncls, q, S = (plan[k] for k in ("B", "G", "Cpfx", "ncls", "q", "n_states"))
    nodes = plan["nodes"]
    devbuf = [int(x) for x in plan["devbuf"]]
    lvals = [0] * ((S - 1) * 2 * q)
    dV = [[0] * Cp for _ in range(B)]
    for b in range(B):
        fen = [0] * Cp
        leaf = dV[b]
        fac = [int(x) for x in plan["fac_start"][b * G:(b + 1) * G]]

        def add(i, v):
            while i <= ncls:
                fen[i] = (fen[i] + v) & MASK
                i += i & -i

        def pref(i):
            r = 0
            while i > 0:
                r += fen[i]
                i -= i & -i
            return r & MASK
        for v in range(int(plan["block_v0"][b]), int(plan["block_v1"][b])):
            p = nodes[v]
            if p["kind"] == 1:
                for side in ("old", "new"):
                    if p["ex_" + side] and p["amt_" + side] != 0:
                        sgn = -1 if side == "old" else 1
                        g, c, amt = int(p["g_" + side]), int(p["c_" + side]), int(p["amt_" + side])
                        wv = sgn * fac[g] * amt
                        leaf[c + 1] = (leaf[c + 1] + wv) & MASK
                        add(c + 1, wv)
                        off = int(plan["need_off"][b * G + g])
                        if off >= 0:
                            ti = int(p["ti_" + side])
                            devbuf[off + ti] = s64(devbuf[off + ti] + sgn * amt)
            elif p["kind"] == 2:
                g = int(p["g_old"])
                ds = int(p["fac_val"]) - int(p["fac_prev"])
                r = int(plan["g2row"][g])
                off = int(plan["need_off"][b * G + g])
                if r >= 0 and ds != 0:
                    for k in range(int(plan["ms_off"][r]), int(plan["ms_off"][r + 1])):
                        di = int(plan["ms_dev"][k])
                        dev = devbuf[off + di] if (di >= 0 and off >= 0) else 0
                        d = ds * (int(plan["ms_base"][k]) + dev)
                        if d:
                            c1 = int(plan["ms_cls"][k]) + 1
                            leaf[c1] = (leaf[c1] + d) & MASK
                            add(c1, d)
                fac[g] = int(p["fac_val"])
            base = (v - 1) * 2 * q
            for kk in range(q):
                lvals[base + 2 * kk] = pref(int(plan["qlb"][v * q + kk]))
                lvals[base + 2 * kk + 1] = pref(int(plan["qhb"][v * q + kk]))
    vstart = [int(x) & MASK for x in plan["vbase"]]
    carry = []
    for b in range(B):
        cp = [0] * Cp
        for k in range(1, Cp):
            cp[k] = (cp[k - 1] + vstart[k]) & MASK
        carry.append(cp)
        for k in range(1, Cp):
            vstart[k] = (vstart[k] + dV[b][k]) & MASK
    ans = []
    for v in range(1, S):
        cp = carry[int(plan["bidx"][v])]
        for kk in range(q):
            i, j = int(plan["qlb"][v * q + kk]), int(plan["qhb"][v * q + kk])
            base = (v - 1) * 2 * q
            ans.append(s64(cp[j] - cp[i] + lvals[base + 2 * kk + 1] - lvals[base + 2 * kk]))
    return (np.array(ans, dtype=np.int64), np.array([[s64(x) for x in row] for row in dV], dtype=np.int64),
            np.array([s64(x) for x in lvals], dtype=np.int64))
