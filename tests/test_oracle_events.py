"""The contact-event restatement (oracle/contact_events.py) on hand-made states: the behaviour
of the reference's ContactWatch (src/vendor/three-avbd-lib/contacts.ts) that the engine's events
are checked against."""
import numpy as np

import contact_events as CE


def _state(pairs, counts, n=6):
    m = len(pairs)
    c = int(np.sum(counts))
    return dict(mpairs=np.array(pairs, dtype=np.uint32).reshape(m, 2), mcount=np.array(counts, dtype=np.int32),
                pos=np.tile([1.0, 2.0, 3.0], (n, 1)), quat=np.tile([0.0, 0.0, 0.0, 1.0], (n, 1)),
                cra=np.tile([0.5, 0.0, 0.0], (c, 1)), clam=np.tile([-10.0, 0.0, 0.0], (c, 1)))


def test_begin_stay_end_and_watch_changes():
    watch = np.ones(6, dtype=np.int64)
    normal = lambda a, b: [0.0, 1.0, 0.0]  # noqa: E731
    s1 = _state([(2, 0), (3, 1)], [2, 0])
    ev, now = CE.step_events(set(), np.zeros(6, dtype=np.int64), s1, watch, 1, 0.5, normal)
    assert [(e[0], e[1], e[2]) for e in ev] == [(CE.BEGIN, 2, 0)] and now == {(2, 0)}
    assert np.allclose(ev[0][4], [1.5, 2.0, 3.0]) and ev[0][5] == 10.0  # mean point on A, |sum lam| dt
    s2 = _state([(2, 0), (3, 1)], [1, 3])
    ev, now2 = CE.step_events(now, watch.copy(), s2, watch, 2, 0.5, normal)
    assert [(e[0], e[1], e[2]) for e in ev] == [(CE.BEGIN, 3, 1)]  # (2, 0) stays: no event
    s3 = _state([(3, 1)], [3])
    ev, now3 = CE.step_events(now2, watch.copy(), s3, watch, 3, 0.5, normal)
    assert [(e[0], e[1], e[2]) for e in ev] == [(CE.END, 2, 0)]
    # a reset (watch word + 2) begins the body's contacts afresh and ends none of the old ones
    w4 = watch.copy()
    w4[1] += 2
    ev, _ = CE.step_events(now3, watch.copy(), _state([], []), w4, 4, 0.5, normal)
    assert ev == []
    ev, _ = CE.step_events(now3, watch.copy(), s3, w4, 4, 0.5, normal)
    assert [(e[0], e[1], e[2]) for e in ev] == [(CE.BEGIN, 3, 1)]
    # unwatched pairs are not touching
    ev, now5 = CE.step_events(set(), np.zeros(6, dtype=np.int64), s2, np.zeros(6, dtype=np.int64), 5, 0.5, normal)
    assert ev == [] and now5 == set()
