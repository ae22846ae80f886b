"""The autotuner's selection logic on the CPU with a stand-in batch."""
from lpmd2_gb300.autotune import CELL_SCALES, LANES_PER_ATOM, SKINS_A, SKINS_SIGMA, tune_batch, tune_skin


class Stub:
    def __init__(self, p, log):
        self.p, self.log, self.closed = p, log, False

    def close(self):
        self.closed = True
        self.log.append(self)


def test_picks_fastest_and_closes_every_trial():
    closed = []
    cost = lambda p: (abs(p["skin_sigma"] - 0.3) * 10 + (0.5 if p["cell_scale"] == 2 else 0.0)  # noqa: E731
                      + abs(p["lanes_per_atom"] - 4) * 0.01)
    best, trials = tune_batch(lambda p: Stub(p, closed), lambda b: 1.0 + cost(b.p))
    assert best == {"skin_sigma": 0.3, "cell_scale": 1, "lanes_per_atom": 4}
    # the skin x cell grid at one lane, then the other lane counts at the best grid point
    assert len(trials) == len(SKINS_SIGMA) * len(CELL_SCALES) + len(LANES_PER_ATOM) - 1 == len(closed)
    assert [t["lanes_per_atom"] for t in trials[-5:]] == [2, 4, 8, 16, 32]
    assert all(t["skin_sigma"] == 0.3 and t["cell_scale"] == 1 for t in trials[-5:])
    assert all(s.closed for s in closed)


def test_trial_failure_still_closes():
    closed = []

    def timing(b):
        raise RuntimeError("boom")

    try:
        tune_batch(lambda p: Stub(p, closed), timing)
    except RuntimeError:
        pass
    assert len(closed) == 1 and closed[0].closed


def test_skin_tuner_picks_fastest_and_closes():
    closed = []
    best, trials = tune_skin(lambda k: Stub({"skin": k}, closed), lambda b: 1.0 + abs(b.p["skin"] - 0.4))
    assert best == 0.4
    assert [t["skin"] for t in trials] == list(SKINS_A) and len(closed) == len(SKINS_A)
    assert all(s.closed for s in closed)

