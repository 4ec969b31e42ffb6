"""The bookkeeping of the range form of the many-body force rows (k_force_rg,
csrc/assemble.cu), restated in Python and checked on the CPU.

* Partition and merge: thread t takes powers [t S, t S + S) of a cluster type; it
  writes every column whose powers all lie in its range, hands the partial sum of a
  column that began in an earlier range to shared memory, and, for a column that
  continues past its range, adds the later threads' partials in thread order.  Every
  column must be written exactly once, with the sum of its powers' values, for the
  column groups (PARAM_INDICES) of every 3- and 4-body type of the C/H/N/O model and
  for random group layouts.
* Tables: the M / Q tables of one cluster built the kernel's way (4-body M from
  (p0, p1) partial products, PERM_SCALE folded into Q) equal the direct per-entry
  products, for every owner role, with the slot roles packed as in dev.cuh.
"""
import importlib
import random

import numpy as np
import pytest


def _groups_from_header(text):
    """Per cluster type: the column (PARAM_INDICES) of each allowed power, in power
    order, from the params.header text (one row per power: index, powers, equivalent
    index, parameter index)."""
    types, cur = [], None
    for line in text.splitlines():
        if line.startswith(" PAIRS:"):
            cur = []
            types.append(cur)
            continue
        t = line.split()
        if cur is not None and t and t[0].isdigit() and len(t) in (6, 9):
            cur.append(int(t[-1]))
    return [t for t in types if t]


def _emulate(tcol, nt, vals):
    n = len(tcol)
    S = (n + nt - 1) // nt
    ncol = max(tcol) + 1
    gstart = [None] * (ncol + 1)
    for p in range(n - 1, -1, -1):
        gstart[tcol[p]] = p
    gstart[ncol] = n
    written, out, part, tails = [0] * ncol, [0.0] * ncol, [None] * nt, []
    for tid in range(nt):
        pb = min(n, tid * S)
        pe = min(n, pb + S)
        head = pb < pe and pb > 0 and tcol[pb - 1] == tcol[pb]
        acc, pcol, first = 0.0, -1, True
        for p in range(pb, pe):
            col = tcol[p]
            if p > pb and col != pcol:
                if first and head:
                    part[tid] = acc
                else:
                    written[pcol] += 1
                    out[pcol] = acc
                first, acc = False, 0.0
            pcol = col
            acc += vals[p]
        if pb < pe:
            ends = pe == n or tcol[pe] != pcol
            if first and head:
                part[tid] = acc
            elif ends:
                written[pcol] += 1
                out[pcol] = acc
            else:
                tails.append((tid, pcol, acc))
    for tid, pcol, acc in tails:
        last = (gstart[pcol + 1] - 1) // S
        assert last < nt
        for t2 in range(tid + 1, last + 1):
            assert part[t2] is not None, (tid, t2)
            acc += part[t2]
        written[pcol] += 1
        out[pcol] = acc
    for c in range(ncol):
        assert written[c] == 1, (c, written[c])
        exp = sum(vals[gstart[c]:gstart[c + 1]])
        assert abs(out[c] - exp) <= 1e-12 * (1 + abs(exp))


@pytest.fixture(scope="module")
def chno_groups(cg, tmp_path_factory):
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload("chno-4b", str(tmp_path_factory.mktemp("chno")), nframes=1, seed=5, labels=False)
    return _groups_from_header(cg.Model(fm).params_header())


def test_column_groups_are_contiguous(chno_groups):
    assert len(chno_groups) == 20 + 35   # triplet and quadruplet types of 4 species
    for tc in chno_groups:
        assert all(a <= b for a, b in zip(tc, tc[1:]))
    assert {len(tc) for tc in chno_groups} == {490, 3861}


@pytest.mark.parametrize("nt", [512, 352, 256, 7, 1])
def test_every_model_column_written_once(chno_groups, nt):
    rng = random.Random(nt)
    for tc in chno_groups:
        _emulate(tc, nt, [rng.random() for _ in tc])


def test_random_group_layouts():
    rng = random.Random(11)
    for _ in range(400):
        n = rng.choice([1, 2, 5, 31, 511, 512, 513, 1000, 3861, 4096])
        tc, c = [], 0
        while len(tc) < n:
            tc += [c] * rng.choice([1, 1, 2, 3, 6, 24, 60])
            c += 1
        _emulate(tc[:n], rng.choice([512, 352, 32, 3, 1]), [rng.random() for _ in range(n)])


def _slot_in(nb, pi, k):
    return (0x212010 >> (4 * (2 * pi + k))) & 15 if nb == 3 else (0x542531430210 >> (4 * (3 * pi + k))) & 15


def _slot_out(nb, pi, k):
    return (0x012 >> (4 * pi)) & 15 if nb == 3 else (0x310420521543 >> (4 * (3 * pi + k))) & 15


def test_packed_role_slots():
    """Incident slots of each canonical position: the edges (pairs of members) that
    contain it; the other slots are the rest."""
    edges = {3: [(0, 1), (0, 2), (1, 2)], 4: [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]}
    for nb, ed in edges.items():
        for pi in range(nb):
            inc = [_slot_in(nb, pi, k) for k in range(nb - 1)]
            out = [_slot_out(nb, pi, k) for k in range(len(ed) - nb + 1)]
            assert inc == [e for e, m in enumerate(ed) if pi in m]
            assert out == [e for e, m in enumerate(ed) if pi not in m]


@pytest.mark.parametrize("nb,order", [(3, 8), (3, 16), (4, 4), (4, 3)])
def test_factored_tables_equal_direct_products(nb, order):
    rng = np.random.default_rng(nb * 100 + order)
    NP = 3 if nb == 3 else 6
    NI, NO = nb - 1, NP - nb + 1
    sizeI, sizeO, perm = order ** NI, order ** NO, 1.0 / 24.0
    for role in range(nb):
        G = rng.standard_normal((NP, order))        # g_s[n]
        W = rng.standard_normal((NP, 3, order))     # owner-weighted h_s[n], x / y / z
        I = [_slot_in(nb, role, u) for u in range(NI)]
        O = [_slot_out(nb, role, u) for u in range(NO)]
        direct = np.zeros(3 * sizeI + sizeO)
        for z in range(sizeI):
            pw = [(z // order ** u) % order for u in range(NI)]
            for c in range(3):
                direct[c * sizeI + z] = sum(W[I[u], c, pw[u]] * np.prod([G[I[v], pw[v]] for v in range(NI) if v != u])
                                            for u in range(NI))
        for z in range(sizeO):
            direct[3 * sizeI + z] = perm * np.prod([G[O[u], (z // order ** u) % order] for u in range(NO)])
        kern = np.zeros_like(direct)
        nzm = order * order if NI == 3 else sizeI
        for z in range(nzm + sizeO):
            if z >= nzm:
                zz, prod = z - nzm, perm
                for u in range(NO):
                    prod *= G[O[u], zz % order]
                    zz //= order
                kern[3 * sizeI + z - nzm] = prod
                continue
            p0, p1 = z % order, z // order % order
            g0, g1, w0, w1 = G[I[0]], G[I[1]], W[I[0]], W[I[1]]
            if NI == 2:
                for c in range(3):
                    kern[c * sizeI + z] = w0[c, p0] * g1[p1] + w1[c, p1] * g0[p0]
            else:
                g2, w2 = G[I[2]], W[I[2]]
                gg = g0[p0] * g1[p1]
                b = [w0[c, p0] * g1[p1] + g0[p0] * w1[c, p1] for c in range(3)]
                for p2 in range(order):
                    for c in range(3):
                        kern[c * sizeI + z + p2 * order * order] = b[c] * g2[p2] + gg * w2[c, p2]
        assert np.abs(kern - direct).max() <= 1e-13 * np.abs(direct).max()
