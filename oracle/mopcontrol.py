"""Oracle restatement of the multi-index control (integer work, bit-exact).

Test infrastructure only (see ``oracle/__init__.py``).

Follows src/mopcontrol.jl:6-241 and src/estimate.jl:1-36 literally, including
the reference's loop quirks (the downward scan in ``add_boundary_modes`` that
keeps the *smallest* nonzero position above the running value, and the
``sleep(1)`` at mopcontrol.jl:74 which is omitted here because it does no
arithmetic).  Multi-indices are Python lists; positions are 0-based where the
reference is 1-based, with the translation noted at each loop.
"""
import copy


def generate_multiindices(M, deg):
    """mopcontrol.jl:6-22 (full tensor set, last dimension fastest)."""
    mis = [[j] for j in range(deg + 1)]
    L = len(mis)
    for _ in range(1, M):
        for i in range(L):
            for j in range(deg + 1):
                new_mi = copy.deepcopy(mis[i])
                new_mi.append(j)
                mis.append(new_mi)
        mis = mis[L:]
        L *= deg + 1
    return mis


def prepare_multi_indices(mis, minimal_length=0):
    """mopcontrol.jl:29-37 (in place)."""
    new_length = max(minimal_length, max(len(mi) for mi in mis))
    for mi in mis:
        while len(mi) < new_length:
            mi.append(0)


def add_boundary_modes(mis, p_extension=1, tail_extension=(10, 2)):
    """mopcontrol.jl:60-132.  Mutates ``mis`` (padding) like the reference."""
    last_nonzero = 0  # 1-based position
    maxdegree1 = 0
    nmodes = len(mis)
    for j in range(1, len(mis)):  # julia j in 2:length
        maxdegree1 = max(maxdegree1, mis[j][0])
        # julia: for k in length(mi):-1:(last_nonzero+1), range fixed at entry
        lo = last_nonzero + 1
        for k in range(len(mis[j]), lo - 1, -1):
            if mis[j][k - 1] != 0:
                last_nonzero = k
    # sleep(1) at mopcontrol.jl:74 omitted (no arithmetic)
    prepare_multi_indices(mis, minimal_length=last_nonzero + tail_extension[0])
    ext = copy.deepcopy(mis)
    maxlength2 = max(len(mi) for mi in ext)

    for k in range(1, maxlength2 + 1):
        new = copy.deepcopy(mis[0])
        new[k - 1] = 1
        if new not in ext:
            ext.append(new)

    for k in range(maxdegree1 + 1, maxdegree1 + p_extension + 1):
        new = copy.deepcopy(mis[0])
        new[0] = k
        if new not in ext:
            ext.append(new)

    for j in range(nmodes):
        last_nonzero_pos = 1
        for k in range(len(mis[j]), 0, -1):
            if mis[j][k - 1] != 0:
                last_nonzero_pos = k
                break
        for k in range(1, last_nonzero_pos + tail_extension[1] + 1):
            if k > last_nonzero + tail_extension[1]:
                break
            new = copy.deepcopy(mis[j])
            new[k - 1] += 1
            if new not in ext:
                ext.append(copy.deepcopy(new))
    return ext


def get_neighbours(mis):
    """estimate.jl:1-22.  Returns PLUS, MINUS as M x nmodes arrays of 1-based
    mode numbers (0 = no neighbour), exactly as the reference stores them."""
    M = len(mis[0])
    n = len(mis)
    plus = [[0] * n for _ in range(M)]
    minus = [[0] * n for _ in range(M)]
    for j in range(n):
        for m in range(M):
            mu1 = list(mis[j])
            mu2 = list(mis[j])
            mu1[m] += 1
            mu2[m] -= 1
            for k in range(n):
                if mis[k] == mu1:
                    plus[m][j] = k + 1
                elif mis[k] == mu2:
                    minus[m][j] = k + 1
    return plus, minus


def classify_modes(mis, active_modes=None):
    """mopcontrol.jl:168-241.  Returns 1-based index lists
    (inactive_else, inactive_bnd, inactive_bnd2, active_bnd, active_int)."""
    if active_modes is None:
        active_modes = mis
    active_bnd, active_int, inactive_bnd, inactive_bnd2, inactive_else = [], [], [], [], []
    new = list(mis[0])
    for j in range(len(mis)):
        last_nonzero_pos = 1
        active = True
        for k in range(len(mis[j]), 0, -1):
            if mis[j][k - 1] != 0:
                last_nonzero_pos = k
                break
        if mis[j] in active_modes:
            if last_nonzero_pos == len(mis[j]):
                active_bnd.append(j + 1)
            else:
                for k in range(1, last_nonzero_pos + 2):
                    new[:] = mis[j]
                    new[k - 1] += 1
                    if new not in active_modes:
                        active = False
                        break
                if active:
                    active_int.append(j + 1)
                else:
                    active_bnd.append(j + 1)
        else:
            bnd_level = 0
            kmax = min(last_nonzero_pos + 1, len(new))
            for k in range(1, kmax + 1):
                new[:] = mis[j]
                if new[k - 1] > 0:
                    new[k - 1] -= 1
                    if new in active_modes:
                        bnd_level = 1
                        inactive_bnd.append(j + 1)
                        break
            if bnd_level == 0:
                done = False
                for k in range(1, kmax + 1):
                    for k2 in range(1, kmax + 1):
                        new[:] = mis[j]
                        if new[k - 1] > 0 and new[k2 - 1] > 0:
                            new[k - 1] -= 1
                            new[k2 - 1] -= 1
                            if new in active_modes:
                                bnd_level = 2
                                inactive_bnd2.append(j + 1)
                                done = True
                                break
                    if done:
                        # julia's `for k in .., k2 in ..` is one loop: break leaves both
                        break
                if bnd_level == 0:
                    inactive_else.append(j + 1)
    return inactive_else, inactive_bnd, inactive_bnd2, active_bnd, active_int


def stable_sortperm_desc(values):
    """Julia ``sortperm(v; rev=true)`` (stable: ties keep ascending index).
    Returns 1-based indices."""
    return [i + 1 for i in sorted(range(len(values)), key=lambda i: (-values[i], i))]


def stochastic_marking(eta4modes, mis_ext, nmodes_active, multi_indices, theta_stochastic=0.5,
                       factor_tail=1.0, zeta_data=0.0):
    """scripts/poisson.jl:341-420: classification, split of the estimator into
    active/tail parts, the spatial-vs-stochastic decision and the Doerfler
    stochastic marking.  Returns (decision, new multi_indices, extra) where
    decision is "spatial" or "stochastic"."""
    inactive_else, inactive_bnd, inactive_bnd2, active_bnd, active_int = classify_modes(
        mis_ext, mis_ext[:nmodes_active])
    sorted_id = stable_sortperm_desc(eta4modes)
    est_int = 0.0
    est_bnd = 0.0
    actives = set(active_int) | set(active_bnd)
    for j in range(len(mis_ext)):
        sid = sorted_id[j]
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
        acc = 0.0
        bnd = set(inactive_bnd) | set(inactive_bnd2)
        for j in range(len(mis_ext)):
            sid = sorted_id[j]
            if sid in bnd:
                acc += eta4modes[sid - 1] ** 2
                new_mis.append(list(mis_ext[sid - 1]))
                added.append(sid)
                if acc >= theta_stochastic * est_bnd:
                    break
    classes = dict(inactive_else=inactive_else, inactive_bnd=inactive_bnd, inactive_bnd2=inactive_bnd2,
                   active_bnd=active_bnd, active_int=active_int)
    return decision, new_mis, dict(sorted_id=sorted_id, est_int=est_int, est_bnd=est_bnd,
                                   added=added, classes=classes, actives=sorted(actives))
