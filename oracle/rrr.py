"""ORACLE (test infrastructure only) -- dense restatement of one process's
RRR contraction over unique-block storage.

RRR stores only canonical blocks (non-increasing block coordinates within a
symmetry group, tensor.cc:617-640) and recovers a flipped block by permuting
the stored one (get_symm_permutation, contraction.cc:132-160) -- with no sign,
i.e. a symmetric tensor.  ``sign=-1`` gives the antisymmetric variant that
coupled-cluster amplitudes need.  The contraction of Contraction::contract
(contraction.cc:2447-2870) computes, for every stored C block, the sum over
the full contracted index ranges; this module expands the stored blocks to
dense arrays, contracts with einsum in FP64, and cuts C's blocks back out.
"""
import itertools

import numpy as np


def groups_of(sym):
    return [0 if c in "aA" else 1 if c in "bB" else -1 for c in sym]


def canonical(addr, groups):
    """Sort block coords non-increasing within each group; returns
    (canonical coords, order) with stored dim s holding virtual dim order[s],
    and the number of transpositions (stable bubble sort)."""
    addr = list(addr)
    order = list(range(len(addr)))
    swaps = 0
    for g in sorted(set(x for x in groups if x >= 0)):
        pos = [d for d in range(len(addr)) if groups[d] == g]
        who = list(pos)
        for i in range(len(pos)):
            for j in range(len(pos) - 1 - i):
                if addr[who[j]] < addr[who[j + 1]]:
                    who[j], who[j + 1] = who[j + 1], who[j]
                    swaps += 1
        for i, p in enumerate(pos):
            order[p] = who[i]
    canon = [addr[order[s]] for s in range(len(addr))]
    return tuple(canon), order, swaps


def dense(tiles, addrs, sym, block_range, vgrid, sign=1):
    """Expand stored blocks (tiles: (n, prod(block_range))) to the dense tensor."""
    groups = groups_of(sym)
    br = list(block_range)
    out = np.zeros([b * v for b, v in zip(br, vgrid)])
    stored = {tuple(a): i for i, a in enumerate(np.asarray(addrs).tolist())}
    for v in itertools.product(*[range(g) for g in vgrid]):
        if v in stored:
            blk = tiles[stored[v]].reshape(br)
            f = 1.0
        else:
            canon, order, swaps = canonical(v, groups)
            if canon not in stored:
                continue
            st = tiles[stored[canon]].reshape(br)
            # virtual dim d is stored dim s with order[s] == d
            src = [order.index(d) for d in range(len(v))]
            blk = np.transpose(st, src)
            f = float(sign) ** swaps
        sl = tuple(slice(c * b, (c + 1) * b) for c, b in zip(v, br))
        out[sl] = f * blk
    return out


def cut(dense_arr, addrs, block_range):
    br = list(block_range)
    res = []
    for a in np.asarray(addrs).tolist():
        sl = tuple(slice(c * b, (c + 1) * b) for c, b in zip(a, br))
        res.append(dense_arr[sl].reshape(-1))
    return np.array(res)


def contract(A, B, C, idxA, idxB, idxC, alpha, sign=1):
    """A, B, C: dicts with tiles, addrs, sym, block_range, vgrid.  Returns C's
    new tiles = old + alpha * sum over contracted indices."""
    labels = sorted(set(idxA.split(",")) | set(idxB.split(",")))
    letter = {l: chr(ord("a") + i) for i, l in enumerate(labels)}
    ea = "".join(letter[l] for l in idxA.split(","))
    eb = "".join(letter[l] for l in idxB.split(","))
    ec = "".join(letter[l] for l in idxC.split(","))
    dA = dense(A["tiles"], A["addrs"], A["sym"], A["block_range"], A["vgrid"], sign)
    dB = dense(B["tiles"], B["addrs"], B["sym"], B["block_range"], B["vgrid"], sign)
    dC = np.einsum(f"{ea},{eb}->{ec}", dA, dB)
    return C["tiles"] + alpha * cut(dC, C["addrs"], C["block_range"])
