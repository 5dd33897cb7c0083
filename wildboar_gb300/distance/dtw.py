"""DTW barycenter averaging on the GPU (wildboar.distance.dtw.dtw_average).

``dtw_average(method="mm")`` follows distance/dtw.py:429-594 and the
majorize-minimize loop of ``_mm_dtw_average`` (:661-690).  Every epoch of
every group runs on the device: the alignment, the traceback and the
z / V sums are ``wb_dtw_average_mm_step`` (csrc/barycenter.cu), which keeps
the reference's order of additions, so the means are bit-identical.  The
cost of an epoch (``np.mean`` of the dtw distances of the new mean) is
reduced on the host with numpy from distances computed on the device: for
dtw between series of equal length the squared distance is the final cell
of the next epoch's alignment (the same recurrence and band), so each epoch
costs one alignment pass; wdtw (whose distance uses other weights than
``wdtw_alignment``) and unequal lengths take a distance pass.

``_mm_average_groups`` runs many groups (the clusters of a KMeans update) in
lockstep: one launch per epoch covers every group that has not converged.
"""

import ctypes
import math
import numbers

import numpy as np

from .. import _lib
from ._distance import InvalidParameterError, pairwise_distance
from ._validation import check_array
from .lb import dtw_envelope as _envelope_rows

_lib.declare(
    "wb_dtw_average_mm_step",
    [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
     ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
     ctypes.c_void_p, ctypes.c_void_p],
)
_lib.declare(
    "wb_dtw_average_ssg_epoch",
    [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
     ctypes.c_void_p, ctypes.c_void_p],
)
_lib.declare(
    "wb_dtw_alignment",
    [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p],
)
_lib.declare(
    "wb_lb_keogh_terms",
    [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
     ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p],
)
_lib.declare(
    "wb_group_mean",
    [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
     ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p],
)


def check_random_state(seed):
    """sklearn.utils.check_random_state: None, an int or a RandomState."""
    if seed is None or seed is np.random:
        return np.random.mtrand._rand
    if isinstance(seed, numbers.Integral) and not isinstance(seed, bool):
        return np.random.RandomState(seed)
    if isinstance(seed, np.random.RandomState):
        return seed
    raise ValueError("%r cannot be used to seed a numpy.random.RandomState instance" % seed)


def _check_scalar(x, name, *, min_val=None, max_val=None, include_min=True, include_max=True):
    if not isinstance(x, numbers.Real) or isinstance(x, bool):
        raise TypeError(f"{name} must be an instance of float, not {type(x).__qualname__}.")
    if min_val is not None and (x < min_val or (not include_min and x == min_val)):
        raise ValueError(f"{name} == {x}, must be {'>=' if include_min else '>'} {min_val}.")
    if max_val is not None and (x > max_val or (not include_max and x == max_val)):
        raise ValueError(f"{name} == {x}, must be {'<=' if include_max else '<'} {max_val}.")
    return x


def jeong_weight(n, g=0.05):
    """Weights of wdtw_alignment (distance/dtw.py:330-359), computed with numpy."""
    return 1.0 / (1.0 + np.exp(-g * (np.arange(n, dtype=float) - n / 2.0)))


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("dtw_average needs a CUDA device (wildboar_gb300 has no CPU path)")
    return torch


def _to_device(a, torch):
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def _layout(groups, active, torch, dev):
    """Pair arrays of the active groups: member, pair_group, group_start, groups."""
    members = [groups[g] for g in active]
    counts = np.array([len(m) for m in members], dtype=np.int64)
    start = np.zeros(len(active) + 1, dtype=np.int64)
    np.cumsum(counts, out=start[1:])
    member = np.concatenate(members).astype(np.int64) if members else np.zeros(0, np.int64)
    pg = np.repeat(np.asarray(active, dtype=np.int32), counts)
    return (torch.as_tensor(member, device=dev), torch.as_tensor(pg, device=dev),
            torch.as_tensor(start, device=dev),
            torch.as_tensor(np.asarray(active, dtype=np.int32), device=dev), start)


def _step(Xd, means, lay, r, wdev, swdev, new_means, last, torch):
    member, pg, gs, gid, _ = lay
    n_groups = gid.shape[0]
    n_pairs = member.shape[0]
    st = _lib.lib().wb_dtw_average_mm_step(
        Xd.data_ptr(), Xd.stride(0), Xd.shape[1], means.data_ptr(), means.shape[1],
        member.data_ptr(), pg.data_ptr(), gs.data_ptr(), gid.data_ptr(), n_groups, n_pairs,
        float(r), None if wdev is None else wdev.data_ptr(),
        None if swdev is None else swdev.data_ptr(),
        None if new_means is None else new_means.data_ptr(),
        None if last is None else last.data_ptr(),
        _lib.current_stream_handle())
    _lib.check(st)


def _group_cost(dist, sample_weight):
    """costfn of dtw_average (distance/dtw.py:552-557) on host distances."""
    if sample_weight is None:
        return np.mean(dist)
    return np.average(dist, weights=sample_weight)


def _mm_average_groups(Xd, groups, init, *, r, g=None, sample_weight=None, tol=1e-5,
                       max_epoch=50, verbose=False):
    """MM barycenters of several groups of rows of the device matrix ``Xd``.

    ``groups[i]`` are row indices of Xd (in the order the reference's group
    array holds them), ``init`` the (n_groups, mean_len) initial means and
    ``sample_weight`` None or one weight array per group.  Returns the means
    (numpy, n_groups x mean_len) and the costs, as ``_mm_dtw_average``
    returns them per group.
    """
    torch = _torch()
    dev = Xd.device
    G = len(groups)
    init = np.ascontiguousarray(init, dtype=np.float64).reshape(G, -1)
    nm, T = init.shape[1], Xd.shape[1]
    cur = torch.as_tensor(init, device=dev).clone()
    nxt = torch.empty_like(cur)
    wdev = None
    metric, metric_params = "dtw", {"r": r}
    if g is not None:
        wdev = torch.as_tensor(jeong_weight(max(nm, T), g), device=dev)
        metric, metric_params = "wdtw", {"r": r, "g": g}
    fused = g is None and nm == T
    sw = [None] * G if sample_weight is None else sample_weight
    costs = np.full(G, np.nan)

    def swdev_of(lay_active):
        if sample_weight is None:
            return None
        return torch.as_tensor(np.concatenate([np.asarray(sw[a], dtype=np.float64)
                                               for a in lay_active]), device=dev)

    def distance_costs(means_t, active):
        out = {}
        for a in active:
            d = pairwise_distance(means_t[a], Xd[torch.as_tensor(groups[a], device=dev)],
                                  metric=metric, metric_params=metric_params)
            d = d.reshape(-1).cpu().numpy() if hasattr(d, "cpu") else np.atleast_1d(d)
            out[a] = _group_cost(d, sw[a])
        return out

    active = list(range(G))
    lay = _layout(groups, active, torch, dev)
    swd = swdev_of(active)
    final = np.empty((G, nm))
    last = torch.empty(lay[0].shape[0], dtype=torch.float64, device=dev) if fused else None

    def fused_costs():
        n_pairs = lay[0].shape[0]
        sq = np.sqrt(last[:n_pairs].cpu().numpy())
        start = lay[4]
        return {a: _group_cost(sq[start[i]:start[i + 1]], sw[a]) for i, a in enumerate(active)}

    if fused:
        # one pass gives the cost of the current means and the next means
        _step(Xd, cur, lay, r, wdev, swd, nxt, last, torch)
        cost = fused_costs()
    else:
        cost = distance_costs(cur, active)
    for epoch in range(max_epoch):
        if not active:
            break
        if fused:
            # the rows of the active groups in nxt are this epoch's means
            cur, nxt = nxt, cur
            _step(Xd, cur, lay, r, wdev, swd, nxt, last, torch)
            new_cost = fused_costs()
        else:
            _step(Xd, cur, lay, r, wdev, swd, cur, None, torch)
            new_cost = distance_costs(cur, active)
        still, finished = [], []
        for a in active:
            prev_cost, cost[a] = cost[a], new_cost[a]
            if abs(prev_cost - cost[a]) < tol:
                if verbose:
                    print(f"Complete at epoch={epoch} with cost={cost[a]}.")
                finished.append(a)
            else:
                still.append(a)
        if finished:
            host = cur.cpu().numpy()
            final[finished] = host[finished]
            active = still
            if active:
                lay = _layout(groups, active, torch, dev)
                swd = swdev_of(active)
    if active:
        host = cur.cpu().numpy()
        final[active] = host[active]
    for a in range(G):
        costs[a] = cost[a]
    return final, costs


def _ssg_dtw_average(Xd, mean, *, r, g, sample_weight, max_epoch, learning_rate, decay,
                     max_stable, verbose, random_state):
    """_ssg_dtw_average (distance/dtw.py:597-658): the shuffles, learning-rate
    schedule, costs and best-mean bookkeeping on the host, every epoch's
    sample loop one call on the device (wb_dtw_average_ssg_epoch)."""
    torch = _torch()
    dev = Xd.device
    N, T = Xd.shape
    nm = mean.shape[0]
    mean_d = torch.as_tensor(np.ascontiguousarray(mean, dtype=np.float64), device=dev).clone()
    wdev = None
    metric, metric_params = "dtw", {"r": r}
    if g is not None:
        wdev = torch.as_tensor(jeong_weight(max(nm, T), g), device=dev)
        metric, metric_params = "wdtw", {"r": r, "g": g}
    sw = None if sample_weight is None else np.ascontiguousarray(sample_weight, np.float64)
    best_mean = None
    order = np.arange(N)
    min_cost = np.inf
    n_stable = 0
    for epoch in range(max_epoch):
        if n_stable > max_stable:
            if verbose:
                print(f"Completed at epoch={epoch} with cost={min_cost}.")
            break
        random_state.shuffle(order)
        lrs = np.empty(N)
        for i in range(N):
            lrs[i] = learning_rate
            if epoch == 0:
                learning_rate = decay**i * learning_rate
        o = np.ascontiguousarray(order, dtype=np.int64)
        st = _lib.lib().wb_dtw_average_ssg_epoch(
            Xd.data_ptr(), Xd.stride(0), T, mean_d.data_ptr(), nm, _lib.ptr(o), _lib.ptr(lrs),
            N, float(r), None if wdev is None else wdev.data_ptr(), _lib.ptr(sw),
            _lib.current_stream_handle())
        _lib.check(st)
        d = pairwise_distance(mean_d, Xd, metric=metric, metric_params=metric_params)
        d = d.reshape(-1).cpu().numpy()
        cost = _group_cost(d, sw)
        if cost < min_cost:
            if verbose:
                print(f"New min cost={cost} at epoch={epoch} with "
                      f"learning_rate={learning_rate}.")
            min_cost = cost
            n_stable = 0
            best_mean = mean_d.cpu().numpy().copy()
        else:
            n_stable += 1
    return best_mean, min_cost


def dtw_average(X, *, r=1.0, g=None, sample_weight=None, init="random", method="mm",
                max_stable=5, learning_rate=0.1, decay=0.9, tol=1e-5, max_epoch=50,
                return_cost=False, verbose=False, random_state=None):
    """Compute the DTW barycenter average (distance/dtw.py:429-594).

    ``method="mm"`` (the majorize-minimize mean, the reference's default and
    the one KMeans uses) and ``method="ssg"`` (the stochastic subgradient mean,
    a sequential per-sample update, distance/dtw.py:597-658) run on the GPU and
    return the reference's bits.
    """
    X = check_array(X, allow_3d=False, ensure_2d=True, dtype=float)
    if X.shape[0] < 2:
        raise ValueError(
            "Found array with %d sample(s) (shape=%r) while a minimum of 2 is required."
            % (X.shape[0], X.shape))
    r = _check_scalar(r, "r", min_val=0.0, max_val=1.0)
    random_state = check_random_state(random_state)
    if isinstance(init, str) and init == "random":
        mean = X[random_state.randint(X.shape[0])].copy()
    elif hasattr(init, "__len__") or hasattr(init, "__array__"):
        mean = np.array(init, dtype=float, copy=True)
    else:
        raise ValueError("init must be array-like or 'random', not %r" % type(init).__qualname__)
    if sample_weight is not None:
        sample_weight = np.asarray(sample_weight, dtype=np.float64)
        if sample_weight.ndim == 0:
            sample_weight = np.full(X.shape[0], float(sample_weight))
        if sample_weight.shape != (X.shape[0],):
            raise ValueError(
                "sample_weight.shape == {}, expected {}!".format(sample_weight.shape,
                                                                  (X.shape[0],)))
    if g is not None:
        g = _check_scalar(g, "g", min_val=0, include_min=False)
    if method not in ("mm", "ssg"):
        raise ValueError("method must be 'mm' or 'ssg', got %r" % method)
    torch = _torch()
    Xd = _to_device(X, torch)
    if method == "ssg":
        mean, cost = _ssg_dtw_average(
            Xd, mean, r=r, g=g, sample_weight=sample_weight, max_epoch=max_epoch,
            learning_rate=learning_rate, decay=decay, max_stable=max_stable, verbose=verbose,
            random_state=random_state)
        return (mean, cost) if return_cost else mean
    means, costs = _mm_average_groups(
        Xd, [np.arange(X.shape[0])], mean.reshape(1, -1), r=r, g=g,
        sample_weight=None if sample_weight is None else [sample_weight], tol=tol,
        max_epoch=max_epoch, verbose=verbose)
    if return_cost:
        return means[0], costs[0]
    return means[0]


# --------------------------------------------------------------------------
# single-pair helpers of distance/dtw.py:38-426


def _compute_warp_size(x_size, r, *, y_size=0):
    """distance/dtw.py:38-40."""
    _check_scalar(r, "r", min_val=0, max_val=1)
    return max(math.floor(max(x_size, y_size) * r), 1)


def _row(x, name):
    x = check_array(x, allow_3d=False, ensure_2d=False, dtype=float, input_name=name)
    return np.ascontiguousarray(np.ravel(x), dtype=np.float64)


def dtw_distance(x, y, *, r=1.0):
    """Dynamic time warping distance of two series (distance/dtw.py:43-67)."""
    return pairwise_distance(_row(x, "x"), _row(y, "y"), metric="dtw", metric_params={"r": r})


def ddtw_distance(x, y, *, r=1.0):
    """Derivative dtw distance (distance/dtw.py:70-94)."""
    return pairwise_distance(_row(x, "x"), _row(y, "y"), metric="ddtw", metric_params={"r": r})


def wdtw_distance(x, y, *, r=1.0, g=0.05):
    """Weighted dtw distance (distance/dtw.py:97-123)."""
    return pairwise_distance(_row(x, "x"), _row(y, "y"), metric="wdtw",
                             metric_params={"r": r, "g": g})


def wddtw_distance(x, y, *, r=1.0, g=0.05):
    """Weighted derivative dtw distance (distance/dtw.py:126-152)."""
    return pairwise_distance(_row(x, "x"), _row(y, "y"), metric="wddtw",
                             metric_params={"r": r, "g": g})


def dtw_envelop(x, *, r=1.0):
    """LB_Keogh envelope (lower, upper) of one series (distance/dtw.py:155-184)."""
    x = _row(x, "x")
    warp = _compute_warp_size(x.shape[0], r)
    if warp == x.shape[0]:
        warp -= 1
    lo, up = _envelope_rows(x.reshape(1, -1), warp)
    return lo[0], up[0]


def dtw_lb_keogh(x, y=None, *, lower=None, upper=None, r=1.0):
    """LB_Keogh of x against y's envelope (or a given one): (bound, cb)
    (distance/dtw.py:187-243)."""
    x = _row(x, "x")
    if y is not None:
        y = _row(y, "y")
        if y.shape[0] != x.shape[0]:
            raise ValueError(
                "x (%d) and y (%d) must have the same number of timesteps"
                % (x.shape[0], y.shape[0]))
        lower, upper = dtw_envelop(y, r=r)
    elif lower is None or upper is None:
        raise ValueError("both y, lower and upper can't be None")
    lower = _row(lower, "lower")
    upper = _row(upper, "upper")
    if lower.shape[0] != upper.shape[0] or lower.shape[0] != x.shape[0]:
        raise ValueError(
            "lower (%d), upper (%d) and x (%d) have the same number of timesteps"
            % (lower.shape[0], upper.shape[0], x.shape[0]))
    cb = np.empty(x.shape[0])
    dist = np.empty(1)
    st = _lib.lib().wb_lb_keogh_terms(_lib.ptr(x), _lib.ptr(lower), _lib.ptr(upper),
                                      x.shape[0], _lib.ptr(cb), _lib.ptr(dist), 0, None)
    _lib.check(st)
    return float(dist[0]), cb


def dtw_alignment(x, y, *, r=1.0, weight=None, out=None):
    """Cumulative cost matrix of dtw (distance/dtw.py:246-290).  Cells off the
    band are +inf (the reference leaves them unset)."""
    x = _row(x, "x")
    y = _row(y, "y")
    warp_size = _compute_warp_size(x.shape[0], r, y_size=y.shape[0])
    if not 0 < warp_size <= max(x.shape[0], y.shape[0]):
        raise ValueError("invalid r")
    if weight is not None:
        weight = _row(weight, "weight")
        if weight.shape[0] != max(x.shape[0], y.shape[0]):
            raise ValueError(
                "weight must have the same size as max(x.size, y.size) %d, got %d"
                % (max(x.shape[0], y.shape[0]), weight.shape[0]))
    if out is None:
        out = np.empty((x.shape[0], y.shape[0]))
    elif out.shape[0] < x.shape[0] or out.shape[1] < y.shape[0]:
        raise ValueError("out has wrong shape, got [%d, %d]" % out.shape)
    res = np.empty((x.shape[0], y.shape[0]))
    st = _lib.lib().wb_dtw_alignment(_lib.ptr(x), x.shape[0], _lib.ptr(y), y.shape[0],
                                     float(r), _lib.ptr(weight), _lib.ptr(res), 0, None)
    _lib.check(st)
    out[:x.shape[0], :y.shape[0]] = res
    return out


def wdtw_alignment(x, y, *, r=1.0, g=0.5, out=None):
    """Weighted dtw cost matrix (distance/dtw.py:293-327)."""
    x = _row(x, "x")
    y = _row(y, "y")
    return dtw_alignment(x, y, r=r, weight=jeong_weight(max(x.shape[0], y.shape[0]), g),
                         out=out)


def dtw_mapping(x=None, y=None, *, alignment=None, r=1, return_index=False):
    """Optimal warping path as a boolean indicator (distance/dtw.py:362-426):
    from the last cell, the argmin of [diag, up, left], the first minimum
    winning."""
    if alignment is None:
        if x is None or y is None:
            raise ValueError("if alignment=None, neither x or y can be None")
        alignment = dtw_alignment(x, y, r=r)
    else:
        alignment = np.asarray(alignment, dtype=float)
        if alignment.ndim != 2:
            raise ValueError("alignment must be a 2-D array")
    indicator = np.zeros(alignment.shape, dtype=bool)
    i = alignment.shape[0] - 1
    j = alignment.shape[1] - 1
    while i > 0 or j > 0:
        indicator[i, j] = True
        option_diag = alignment[i - 1, j - 1] if i > 0 and j > 0 else np.inf
        option_up = alignment[i - 1, j] if i > 0 else np.inf
        option_left = alignment[i, j - 1] if j > 0 else np.inf
        move = int(np.argmin([option_diag, option_up, option_left]))
        if move == 0:
            i -= 1
            j -= 1
        elif move == 1:
            i -= 1
        else:
            j -= 1
    indicator[0, 0] = True
    if return_index:
        return indicator, indicator.nonzero()
    return indicator


__all__ = ["dtw_average", "jeong_weight", "check_random_state", "InvalidParameterError",
           "dtw_distance", "ddtw_distance", "wdtw_distance", "wddtw_distance", "dtw_envelop",
           "dtw_lb_keogh", "dtw_alignment", "wdtw_alignment", "dtw_mapping"]
