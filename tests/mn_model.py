"""Model of the word positions k_multinomial reads (MnLayout, gr_mv.cuh),
applied to a raw engine word stream.  The CPU tests check it against the
oracle's literal restatement of MultinomialGen::generate, which pins the
kernel's index arithmetic without a GPU."""
import numpy as np


def layout(trials, c0):
    nP, ns = trials >> 2, trials & 3
    W0 = 8 * ((nP + 1) // 2 + ns)
    W1 = 8 * (nP // 2 + ns)
    spu = 2 if nP & 1 else 1
    return dict(nP=nP, ns=ns, W0=W0, W1=W1, spu=spu, c0=c0)


def state(L, i):
    return L["c0"] ^ (i & 1) if L["spu"] == 2 else L["c0"]


def base(L, i):
    if L["spu"] == 1:
        return i * (L["W1"] if L["c0"] else L["W0"])
    return (i >> 1) * (L["W0"] + L["W1"]) + ((L["W1"] if L["c0"] else L["W0"]) if i & 1 else 0)


def cache_off(L, c):
    return 4 * L["nP"] if c == 0 else 4 * L["nP"] - 4


def scalar_off(L, c):
    return 8 * ((L["nP"] + 1) // 2) if c == 0 else 8 * (L["nP"] // 2)


def _i32(x):
    return int(np.int64(x) - (1 << 32) if x & 0x80000000 else x)


def packet_cat(rx, table):
    if table[0] == "cdf":
        cdf = table[1]
        x = rx & 0x7FFFFFFF
        r = len(cdf) - 1
        for c in cdf[:-1]:
            r -= 1 if x < _i32(int(c)) else 0
        return r
    _, prob, alias, mask = table
    a = rx & mask
    return a if (rx >> 1) < prob[a] else int(alias[a])


def scalar_cat(rx, table):
    x = _i32(rx)
    if table[0] == "cdf":
        v = x & 0x7FFFFFFF
        return int(sum(1 for c in table[1][:-1] if int(c) < v))
    _, prob, alias, mask = table
    a = x & mask
    alx = (x >> 1) & 0xFFFFFFFF
    return a if alx < (int(prob[a]) & 0xFFFFFFFF) else int(alias[a])


def counts(words, trials, dim, samples, c0, cache_cats, table):
    """Returns (counts (samples, dim), final state, final cached categories, words used)."""
    L = layout(trials, c0)
    out = np.zeros((samples, dim), np.int64)
    for i in range(samples):
        c = state(L, i)
        b0 = base(L, i)
        for t in range(trials):
            if t < 4 * L["nP"]:
                kk, e = t >> 2, t & 3
                if c == 0:
                    cat = packet_cat(int(words[b0 + 4 * kk + e]), table)
                elif kk == 0:
                    if i > 0:
                        cw = base(L, i - 1) + cache_off(L, state(L, i - 1))
                        cat = packet_cat(int(words[cw + e]), table)
                    else:
                        cat = cache_cats[e]
                else:
                    cat = packet_cat(int(words[b0 + 4 * (kk - 1) + e]), table)
            else:
                cat = scalar_cat(int(words[b0 + scalar_off(L, c) + 8 * (t - 4 * L["nP"])]), table)
            out[i, cat] += 1
    cf = state(L, samples) if L["nP"] > 0 else c0
    cats = list(cache_cats)
    if L["nP"] > 0 and cf == 1 and samples > 0:
        cw = base(L, samples - 1) + cache_off(L, state(L, samples - 1))
        cats = [packet_cat(int(words[cw + e]), table) for e in range(4)]
    return out, cf, cats, base(L, samples)
