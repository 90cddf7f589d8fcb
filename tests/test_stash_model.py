"""The collision stash's bookkeeping (warp_loop_stash in
loki-mc_gb300/csrc/lgpu_advance.cuh), replayed on the host with random
events: every record index the warp reads or writes stays inside the 64
records, the pending stack [0, np) and the ready stack [np, np + nr) never
overlap, np + nr never exceeds 63, and no electron is lost or duplicated.

The model follows the loop step by step: refill (ready records from the top
of the ready stack, then queued secondaries, then the ensemble chunk), the
collision turn (np >= 32, or pending records and no lane flying: lanes
flying an electron take the lowest of the top min(np, 32) pending records
and leave theirs in place, empty lanes take the rest), the flight turn
(each lane finishes, keeps flying after a null collision, or draws a
collision), and the exchange of a pending lane's electron with a ready
record in place."""
import numpy as np
import pytest

NS = 64


def run(seed, n_electrons, p_pend, p_finish, p_ion, p_att):
    rng = np.random.default_rng(seed)
    lanes = [None] * 32  # electron id or None
    stash = [None] * NS  # record slot -> electron id
    np_, nr = 0, 0
    queue = []
    next_id = 0
    exhausted = False
    done = set()
    sec_id = 10 ** 9
    steps = 0

    def check():
        assert 0 <= np_ and 0 <= nr and np_ + nr <= NS - 1
        for e in range(NS):
            occupied = stash[e] is not None
            assert occupied == (e < np_ + nr), (e, np_, nr)
        ids = [x for x in lanes if x is not None] + [x for x in stash if x is not None] + queue
        assert len(ids) == len(set(ids))

    while True:
        steps += 1
        assert steps < 10 ** 6
        # refill: ready records from the top of the ready stack
        need = [i for i in range(32) if lanes[i] is None]
        if need and nr > 0:
            take = min(len(need), nr)
            for r, i in enumerate(need[:take]):
                e = np_ + nr - 1 - r
                assert np_ <= e < np_ + nr
                lanes[i], stash[e] = stash[e], None
            nr -= take
        need = [i for i in range(32) if lanes[i] is None]
        # the warp's queued secondaries
        while need and queue:
            lanes[need.pop(0)] = queue.pop()
        # the ensemble chunk
        for i in need:
            if next_id < n_electrons:
                lanes[i] = next_id
                next_id += 1
            else:
                exhausted = True
        live = [i for i in range(32) if lanes[i] is not None]
        check()
        # collision turn
        if np_ >= 32 or (np_ > 0 and not live):
            k, h = min(np_, 32), len(live)
            order = live + [i for i in range(32) if lanes[i] is None]
            taken = []
            for rank, i in enumerate(order[:k]):
                e = np_ - k + rank
                assert 0 <= e < np_
                lanes[i], stash[e] = stash[e], lanes[i]
                taken.append(i)
            np_ -= k
            nr += min(k, h)
            for i in taken:  # the collision: attachment ends the electron, ionization queues a secondary
                u = rng.random()
                if u < p_att:
                    done.add(lanes[i])
                    lanes[i] = None
                elif u < p_att + p_ion:
                    queue.append(sec_id)
                    sec_id += 1
            check()
            continue
        if not live:
            if exhausted and not queue:
                break
            continue
        # flight turn
        pend = []
        for i in live:
            u = rng.random()
            if u < p_finish:
                done.add(lanes[i])
                lanes[i] = None
            elif u < p_finish + p_pend:
                pend.append(i)
        # a pending lane exchanges its electron with record np + r in place
        k = len(pend)
        for r, i in enumerate(pend):
            e = np_ + r
            assert e < NS
            if r < nr:
                lanes[i], stash[e] = stash[e], lanes[i]
            else:
                assert stash[e] is None
                stash[e], lanes[i] = lanes[i], None
        np_ += k
        nr = max(nr - k, 0)
        check()
    assert np_ == 0 and nr == 0 and not queue
    assert set(range(n_electrons)) <= done
    return steps


@pytest.mark.parametrize("p_pend,p_finish,p_ion,p_att", [
    (0.07, 0.47, 0.0, 0.0),    # the sweep's mix: ~2 events per electron, 15 % of trials real
    (0.5, 0.2, 0.0, 0.0),      # collision-heavy
    (1.0, 0.0, 0.0, 0.05),     # thermal targets: every event goes through the stash (ended by attachment)
    (0.3, 0.3, 0.2, 0.05),     # ionization and attachment
    (0.9, 0.05, 0.2, 0.3),     # frequent ionization and attachment (fewer secondaries than electrons end)
])
def test_stash_bookkeeping_stays_in_bounds(p_pend, p_finish, p_ion, p_att):
    for seed in range(3):
        run(seed, 2000, p_pend, p_finish, p_ion, p_att)
