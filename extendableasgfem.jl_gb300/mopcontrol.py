"""Multi-index control (host side, integer work).

Mirrors src/mopcontrol.jl and src/estimate.jl:1-36 of ExtendableASGFEM.jl with
hash-based membership tests instead of linear searches; every routine keeps
the reference's iteration order and quirks, so the resulting index lists are
identical:
  generate_multiindices     mopcontrol.jl:6-22
  prepare_multi_indices     mopcontrol.jl:29-37
  add_boundary_modes        mopcontrol.jl:60-132 (the downward scan that sets
                            last_nonzero to the smallest nonzero position above
                            its previous value; the sleep(1) at :74 is omitted)
  classify_modes            mopcontrol.jl:168-241
  get_neighbours            estimate.jl:1-22
Stochastic Doerfler marking of scripts/poisson.jl:341-420 is `stochastic_marking`.
"""
import functools
import heapq
import math


def generate_multiindices(M, deg):
    """Full tensor set {0..deg}^M, last dimension varying fastest."""
    mis = [[j] for j in range(deg + 1)]
    for _ in range(1, M):
        mis = [mi + [j] for mi in mis for j in range(deg + 1)]
    return mis


def total_degree_multiindices(M, deg):
    """Total-degree set sum(mu) <= deg: generate_multiindices order (the
    members of the tensor set with sum <= deg, enumerated directly with the
    running sum pruned instead of filtering (deg+1)^M candidates), stably
    sorted by total degree (the zero index first)."""
    mis = []
    cur = [0] * M

    def rec(d, rem):
        if d == M:
            mis.append(list(cur))
            return
        for j in range(min(deg, rem) + 1):
            cur[d] = j
            rec(d + 1, rem - j)
        cur[d] = 0

    rec(0, deg)
    return sorted(mis, key=sum)


def top_weight_multiindices(M, P, decay_factors):
    """The P multi-indices with the largest weights prod_m d_m^mu_m.

    Ties (log-weights equal to 1e-12) are broken by total degree ascending,
    then lexicographically descending; for the cosine coefficient
    d_m = c m^-2 and M = 20, P = 150 the 150th and 151st weights tie.
    """
    logd = [math.log(v) for v in decay_factors[:M]]
    rel = 1e-12

    def logw(mu):
        return sum(k * l for k, l in zip(mu, logd))

    def cmp(a, b):
        la, lb = logw(a), logw(b)
        if abs(la - lb) > rel:  # not a tie: larger weight first
            return -1 if la > lb else 1
        da, db = sum(a), sum(b)
        if da != db:
            return -1 if da < db else 1
        return -1 if tuple(a) > tuple(b) else (1 if tuple(a) < tuple(b) else 0)

    # best-first search: pops come in non-increasing weight; stop once P are
    # popped and the next candidate is strictly lighter than the P-th
    start = tuple([0] * M)
    heap = [(-logw(start), start)]
    seen = {start}
    popped = []
    while heap:
        if len(popped) >= P and -heap[0][0] < logw(popped[P - 1]) - rel:
            break
        _, mu = heapq.heappop(heap)
        popped.append(mu)
        for m in range(M):
            nu = list(mu)
            nu[m] += 1
            nu = tuple(nu)
            if nu not in seen:
                seen.add(nu)
                heapq.heappush(heap, (-logw(nu), nu))
    popped.sort(key=functools.cmp_to_key(cmp))
    return [list(mu) for mu in popped[:P]]


def prepare_multi_indices(mis, minimal_length=0):
    new_length = max(minimal_length, max(len(mi) for mi in mis))
    for mi in mis:
        mi.extend([0] * (new_length - len(mi)))


def _last_nonzero_pos(mi):
    for k in range(len(mi), 0, -1):
        if mi[k - 1] != 0:
            return k
    return 1


def add_boundary_modes(mis, p_extension=1, tail_extension=(10, 2)):
    """Extended multi-index set; mutates `mis` (padding) like the reference."""
    last_nonzero = 0
    maxdegree1 = 0
    nmodes = len(mis)
    for j in range(1, nmodes):
        maxdegree1 = max(maxdegree1, mis[j][0])
        lo = last_nonzero + 1
        for k in range(len(mis[j]), lo - 1, -1):
            if mis[j][k - 1] != 0:
                last_nonzero = k
    prepare_multi_indices(mis, minimal_length=last_nonzero + tail_extension[0])
    ext = [list(mi) for mi in mis]
    present = {tuple(mi) for mi in ext}

    def push(new):
        t = tuple(new)
        if t not in present:
            present.add(t)
            ext.append(list(new))

    L = max(len(mi) for mi in ext)
    for k in range(L):
        new = list(mis[0])
        new[k] = 1
        push(new)
    for k in range(maxdegree1 + 1, maxdegree1 + p_extension + 1):
        new = list(mis[0])
        new[0] = k
        push(new)
    for j in range(nmodes):
        lnz = _last_nonzero_pos(mis[j])
        for k in range(1, lnz + tail_extension[1] + 1):
            if k > last_nonzero + tail_extension[1]:
                break
            new = list(mis[j])
            new[k - 1] += 1
            push(new)
    return ext


def get_neighbours(mis):
    """PLUS[m][j], MINUS[m][j]: 1-based index of mis[j] +/- e_m, 0 if absent."""
    M = len(mis[0])
    n = len(mis)
    index = {}
    for k, mi in enumerate(mis):
        index[tuple(mi)] = k + 1  # the reference keeps the last match
    plus = [[0] * n for _ in range(M)]
    minus = [[0] * n for _ in range(M)]
    get = index.get
    for j, mi in enumerate(mis):
        t = tuple(mi)
        for m in range(M):
            head, k, tail = t[:m], t[m], t[m + 1:]
            plus[m][j] = get(head + (k + 1,) + tail, 0)
            if k > 0:
                minus[m][j] = get(head + (k - 1,) + tail, 0)
    return plus, minus


def classify_modes(mis, active_modes=None):
    """(inactive_else, inactive_bnd, inactive_bnd2, active_bnd, active_int), 1-based."""
    if active_modes is None:
        active_modes = mis
    active = {tuple(mi) for mi in active_modes}
    a_bnd, a_int, i_bnd, i_bnd2, i_else = [], [], [], [], []
    for j, mi in enumerate(mis):
        lnz = _last_nonzero_pos(mi)
        if tuple(mi) in active:
            if lnz == len(mi):
                a_bnd.append(j + 1)
                continue
            interior = True
            for k in range(1, lnz + 2):
                new = list(mi)
                new[k - 1] += 1
                if tuple(new) not in active:
                    interior = False
                    break
            (a_int if interior else a_bnd).append(j + 1)
        else:
            kmax = min(lnz + 1, len(mi))
            level = 0
            for k in range(1, kmax + 1):
                if mi[k - 1] > 0:
                    new = list(mi)
                    new[k - 1] -= 1
                    if tuple(new) in active:
                        level = 1
                        break
            if level == 1:
                i_bnd.append(j + 1)
                continue
            for k in range(1, kmax + 1):
                for k2 in range(1, kmax + 1):
                    if mi[k - 1] > 0 and mi[k2 - 1] > 0:
                        new = list(mi)
                        new[k - 1] -= 1
                        new[k2 - 1] -= 1
                        if tuple(new) in active:
                            level = 2
                            break
                if level == 2:
                    break
            (i_bnd2 if level == 2 else i_else).append(j + 1)
    return i_else, i_bnd, i_bnd2, a_bnd, a_int


def stochastic_marking(eta4modes, mis_ext, nmodes_active, multi_indices, theta_stochastic=0.5,
                       factor_tail=1.0, zeta_data=0.0):
    """scripts/poisson.jl:341-420: returns (decision, new multi-indices, info)."""
    i_else, i_bnd, i_bnd2, a_bnd, a_int = classify_modes(mis_ext, mis_ext[:nmodes_active])
    order = sorted(range(len(eta4modes)), key=lambda i: (-eta4modes[i], i))  # stable sortperm(rev=true)
    sorted_id = [i + 1 for i in order]
    actives = set(a_int) | set(a_bnd)
    est_int = 0.0
    est_bnd = 0.0
    for sid in sorted_id:
        if sid in actives:
            est_int += eta4modes[sid - 1] ** 2
        else:
            est_bnd += eta4modes[sid - 1] ** 2
    new_mis = [list(mi) for mi in multi_indices]
    added = []
    if est_int > factor_tail * est_bnd + zeta_data:
        decision = "spatial"
    else:
        decision = "stochastic"
        bnd = set(i_bnd) | set(i_bnd2)
        acc = 0.0
        for sid in sorted_id:
            if sid in bnd:
                acc += eta4modes[sid - 1] ** 2
                new_mis.append(list(mis_ext[sid - 1]))
                added.append(sid)
                if acc >= theta_stochastic * est_bnd:
                    break
    info = dict(sorted_id=sorted_id, est_int=est_int, est_bnd=est_bnd, added=added, actives=sorted(actives),
                classes=dict(inactive_else=i_else, inactive_bnd=i_bnd, inactive_bnd2=i_bnd2, active_bnd=a_bnd,
                             active_int=a_int))
    return decision, new_mis, info
