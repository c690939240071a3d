"""Expands charge-group pairs into the reference's atom-pair list records.

The engine stores near charge-group pairs (both directions); the reference
stores atom-pair records (nbpplist_lrf src/md.f90:8095-8166, nbpwlist_lrf
9389-9406, nbwwlist_lrf 10987-11000).  This test helper applies the
reference's atom-level rules to the engine's group pairs so both can be
compared as sets of (min(i,j), max(i,j), LJcod).
"""
import numpy as np


def _all_zero(s, i, j):
    ti, tj = s.iac[i], s.iac[j]
    c = s.ljcod[ti, tj]
    return (s.crg[i] * s.crg[j] == 0.0 and s.avdw[ti, c - 1] * s.avdw[tj, c - 1] == 0.0
            and s.bvdw[ti, c - 1] * s.bvdw[tj, c - 1] == 0.0)


def expand(s, group_pairs):
    """Atom-pair records {'pp','pw','ww'} from unordered group pairs."""
    ex = set(map(tuple, np.asarray(s.excl_pairs).reshape(-1, 2).tolist()))
    p14 = set(map(tuple, np.asarray(s.pairs14).reshape(-1, 2).tolist()))
    ljcod = np.asarray(s.ljcod)
    ns, ncs = s.nat_solute, s.ncgp_solute
    out = {"pp": [], "pw": [], "ww": []}
    members = [s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1] for g in range(len(s.cgp_first))]
    isq = np.asarray(s.iqatom) >= 0

    def pp_pairs(ga, gb, same):
        for i in members[ga]:
            if isq[i]:
                continue
            for j in members[gb]:
                if same and i >= j:
                    continue
                if isq[j] or _all_zero(s, i, j):
                    continue
                key = (min(i, j), max(i, j))
                if key in ex:
                    continue
                lj = 3 if key in p14 else int(ljcod[s.iac[i], s.iac[j]])
                out["pp"].append((key[0], key[1], lj))

    for g in range(ncs):
        if not s.excl[s.cgp_switch[g]]:
            pp_pairs(g, g, True)
    for g1, g2 in np.asarray(group_pairs).tolist():
        w1, w2 = g1 >= ncs, g2 >= ncs
        if w1 and w2:
            a, b = s.cgp_switch[g1], s.cgp_switch[g2]
            for la in range(3):
                for ka in range(3):
                    i, j = a + la, b + ka
                    out["ww"].append((min(i, j), max(i, j), int(ljcod[s.iac[ns + la], s.iac[ns + ka]])))
        elif w1 or w2:
            sg, wg = (g2, g1) if w1 else (g1, g2)
            o = s.cgp_switch[wg]
            for i in members[sg]:
                if isq[i]:
                    continue
                for j in (o, o + 1, o + 2):
                    if _all_zero(s, i, j):
                        continue
                    out["pw"].append((min(i, j), max(i, j), int(ljcod[s.iac[i], s.iac[j]])))
        else:
            pp_pairs(g1, g2, False)
    return out


def oracle_records(o, name):
    rec = o.get_list(name)
    return [(min(i, j), max(i, j), int(lj)) for i, j, lj in rec.tolist()]
