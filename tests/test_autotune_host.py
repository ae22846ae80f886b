"""The autotuner's selection logic on the CPU with a stand-in batch."""
from lpmd2_gb300.autotune import CELL_SCALES, SKINS_SIGMA, tune_batch


class Stub:
    def __init__(self, p, log):
        self.p, self.log, self.closed = p, log, False

    def close(self):
        self.closed = True
        self.log.append(self)


def test_picks_fastest_and_closes_every_trial():
    closed = []
    cost = lambda p: abs(p["skin_sigma"] - 0.3) * 10 + (0.5 if p["cell_scale"] == 2 else 0.0)  # noqa: E731
    best, trials = tune_batch(lambda p: Stub(p, closed), lambda b: 1.0 + cost(b.p))
    assert best == {"skin_sigma": 0.3, "cell_scale": 1}
    assert len(trials) == len(SKINS_SIGMA) * len(CELL_SCALES) == len(closed)
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
