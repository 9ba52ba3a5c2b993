"""The grouping of the grouped batched kernels (host logic, no GPU): groups
partition the batch, hold at most 32 particles that share start time,
direction and the presence of non-gravitational parameters, sit in one
perihelion bucket, are ordered inside it by length, eccentricity and then by
the time of pericentre passage, and are queued most expensive first; the
encounter ratio raises a group's place in the queue."""
import numpy as np
import pytest

GM = 2.9591220828411951e-04


def _pop(n=3000, seed=0):
    rng = np.random.default_rng(seed)
    a = rng.uniform(1.0, 3.5, n)
    e = rng.uniform(0.0, 0.4, n)
    M = rng.uniform(0, 2 * np.pi, n)
    inc = rng.uniform(0, 0.3, n)
    # planar-ish Kepler states about a Sun at the origin
    E = M.copy()
    for _ in range(50):
        E = E - (E - e * np.sin(E) - M) / (1 - e * np.cos(E))
    r = a * (1 - e * np.cos(E))
    x = a * (np.cos(E) - e); y = a * np.sqrt(1 - e * e) * np.sin(E)
    nmot = np.sqrt(GM / a ** 3)
    vx = -a * nmot * np.sin(E) / (1 - e * np.cos(E)); vy = a * nmot * np.sqrt(1 - e * e) * np.cos(E) / (1 - e * np.cos(E))
    st = np.stack([x, y * np.cos(inc), y * np.sin(inc), vx, vy * np.cos(inc), vy * np.sin(inc)], axis=1)
    t0 = np.where(rng.uniform(size=n) < 0.8, 8000.0, 8100.0)
    L = np.where(rng.uniform(size=n) < 0.9, 365.25, rng.uniform(30, 900, n))
    te = t0 + np.where(rng.uniform(size=n) < 0.85, L, -L)
    L = np.abs(te - t0)
    prm = np.zeros((n, 3)); ng = rng.uniform(size=n) < 0.1
    prm[ng, 0] = 1e-10
    tp = np.where(te >= t0, (2 * np.pi - M) / nmot, M / nmot)
    q = a * (1 - e)
    # the bucket distance: q, or for an interval shorter than half an orbit
    # without a pericentre passage the smaller heliocentric distance of its ends
    M1 = np.mod(M + np.where(te >= t0, 1.0, -1.0) * nmot * L, 2 * np.pi)
    E1 = M1.copy()
    for _ in range(60):
        E1 = E1 - (E1 - e * np.sin(E1) - M1) / (1 - e * np.cos(E1))
    r1 = a * (1 - e * np.cos(E1))
    short = (tp > L) & (L * nmot < np.pi)
    dist = np.where(short, np.minimum(r, r1), q)
    # the key after length inside a bucket: time to the pericentre passage,
    # or for those short intervals the end at the smaller distance
    k2 = np.where(short, np.where(r1 < r, L, 0.0), tp)
    return t0, te, st, prm, k2, dist


def test_groups_partition_and_share_class():
    from assist_gb300 import batch
    t0, te, st, prm, tp, q = _pop()
    order, groups = batch.group_plan(t0, te, st, params=prm)
    n = t0.size
    assert sorted(order.tolist()) == list(range(n))
    allm = np.concatenate(groups)
    assert sorted(allm.tolist()) == list(range(n))
    bucket = np.floor(8 * np.log2(q ** 1.5))
    for g in groups:
        assert 1 <= g.size <= 32
        assert np.all(t0[g] == t0[g[0]])
        assert np.all((te[g] >= t0[g]) == (te[g[0]] >= t0[g[0]]))
        assert np.all((prm[g, 0] != 0) == (prm[g[0], 0] != 0))
        assert np.all(bucket[g] == bucket[g[0]])


def test_order_inside_a_bucket():
    """group_order 2: within one class the order is length (sixteenth
    octaves, longest first), then time to pericentre passage."""
    from assist_gb300 import batch
    t0, te, st, prm, tp, q = _pop(seed=1)
    order, groups = batch.group_plan(t0, te, st, params=prm, group_order=2)
    L = np.abs(te - t0)
    lbin = -np.floor(16 * np.log2(np.maximum(L, 1e-3)))
    bucket = np.floor(8 * np.log2(q ** 1.5))
    cls = np.stack([t0, (te < t0).astype(float), (prm[:, 0] != 0).astype(float), bucket], axis=1)
    o = order
    same = np.all(cls[o[1:]] == cls[o[:-1]], axis=1)
    k = np.stack([lbin[o], tp[o]], axis=1)
    for i in np.nonzero(same)[0]:
        a, b = k[i], k[i + 1]
        assert a[0] < b[0] or (a[0] == b[0] and a[1] <= b[1] * (1 + 1e-12) + 1e-9), (i, a, b)


def test_order_with_eccentricity_key():
    """The default grouping: inside a class, length bins, then eccentricity
    in eighths, then time to pericentre passage."""
    from assist_gb300 import batch
    t0, te, st, prm, tp, q = _pop(seed=4)
    order, groups = batch.group_plan(t0, te, st, params=prm)
    n = t0.size
    assert sorted(order.tolist()) == list(range(n)) and sorted(np.concatenate(groups).tolist()) == list(range(n))
    r = np.linalg.norm(st[:, :3], axis=1); v2 = (st[:, 3:] ** 2).sum(1); rv = (st[:, :3] * st[:, 3:]).sum(1)
    ecc = np.linalg.norm(((v2 - GM / r)[:, None] * st[:, :3] - rv[:, None] * st[:, 3:]) / GM, axis=1)
    L = np.abs(te - t0)
    lbin = -np.floor(16 * np.log2(np.maximum(L, 1e-3)))
    ebin = np.floor(8 * np.clip(ecc, 0, 0.999))
    bucket = np.floor(8 * np.log2(q ** 1.5))
    cls = np.stack([t0, (te < t0).astype(float), (prm[:, 0] != 0).astype(float), bucket], axis=1)
    o = order
    same = np.all(cls[o[1:]] == cls[o[:-1]], axis=1)
    k = np.stack([lbin[o], ebin[o], tp[o]], axis=1)
    bad = 0
    for i in np.nonzero(same)[0]:
        a, b = k[i], k[i + 1]
        ok = (a[0] < b[0]) or (a[0] == b[0] and (a[1] < b[1] or (a[1] == b[1] and a[2] <= b[2] * (1 + 1e-12) + 1e-9)))
        bad += not ok
    # an eccentricity within a rounding of an eighth can land in either bin
    assert bad <= 2, bad


def _q(st):
    r = np.linalg.norm(st[:, :3], axis=1); v2 = (st[:, 3:] ** 2).sum(1); rv = (st[:, :3] * st[:, 3:]).sum(1)
    ev = ((v2 - GM / r)[:, None] * st[:, :3] - rv[:, None] * st[:, 3:]) / GM
    ecc = np.linalg.norm(ev, axis=1)
    inv_a = 2 / r - v2 / GM
    return (1 - ecc) / inv_a


def test_queue_is_cost_ordered_and_ratio_moves_groups_forward():
    from assist_gb300 import batch
    t0, te, st, prm, tp, _ = _pop(seed=2)
    q = _q(st)
    L = np.abs(te - t0)
    base = L * q ** -0.6
    _, groups = batch.group_plan(t0, te, st, params=prm)
    cost = [base[g].max() for g in groups]
    assert all(cost[i] >= cost[i + 1] * (1 - 1e-9) for i in range(len(cost) - 1))
    # an encounter ratio of 100 on one cheap particle puts its group first
    cheap = int(np.argmin(base))
    ratio = np.zeros(t0.size, np.float32); ratio[cheap] = 100.0
    _, g2 = batch.group_plan(t0, te, st, params=prm, ratio=ratio)
    assert cheap in set(g2[0].tolist())


def test_group_plan_rejects_bad_arguments():
    from assist_gb300 import batch
    t0, te, st, prm, tp, q = _pop(n=10)
    with pytest.raises(RuntimeError):
        batch.group_plan(t0, te, st, group_order=7)
    order, groups = batch.group_plan(t0[:0], te[:0], st[:0])
    assert order.size == 0 and groups == []
    bad = t0.copy(); bad[3] = np.nan
    with pytest.raises(RuntimeError):
        batch.group_plan(bad, te, st)


def test_group_plan_edge_cases():
    """One particle; zero-length and backward intervals; unbound and
    non-finite states (finite times) all form valid groups."""
    from assist_gb300 import batch
    t0, te, st, prm, k2, dist = _pop(n=200, seed=4)
    order, groups = batch.group_plan(t0[:1], te[:1], st[:1])
    assert order.tolist() == [0] and [g.tolist() for g in groups] == [[0]]
    st2 = st.copy()
    st2[0, 3:] *= 5.0                       # hyperbolic
    st2[1] = np.nan                         # non-finite state
    st2[2, :3] = 0.0                        # at the origin
    te2 = te.copy(); te2[3] = t0[3]         # zero length
    order, groups = batch.group_plan(t0, te2, st2, params=prm)
    assert sorted(np.concatenate(groups).tolist()) == list(range(200))
    assert all(1 <= g.size <= 32 for g in groups)
    # the queue is a permutation of the groups in both group orders
    order1, groups1 = batch.group_plan(t0, te2, st2, params=prm, group_order=1)
    assert sorted(np.concatenate(groups1).tolist()) == list(range(200))
