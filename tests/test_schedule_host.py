"""Host logic of the EMA rebuild predictor (pairs_gb300.schedule.EMASchedule), the
trivial policy the learned schedule is measured against: cycle lengths from list build
to the first guard trip are averaged (alpha 0.3); a cycle that ended at a proactive
rebuild before any trip only bounds its length from below, so it can raise the average
but never lower it."""
import pytest

pytest.importorskip("torch")

from pairs_gb300.schedule import EMASchedule  # noqa: E402


def cycle(s, start, trip=None, end=None):
    s.open_cycle(start)
    s.close_cycle(trip, end)


def test_trips_average_with_alpha():
    s = EMASchedule(engine=None, alpha=0.3)
    assert not s.trained and s.predicted() is None
    cycle(s, 0, trip=6)
    assert s.predicted() == 6
    cycle(s, 6, trip=14)                      # length 8
    assert s.predicted() == pytest.approx(0.7 * 6 + 0.3 * 8)
    s.train()
    assert s.trained and s.predicted_steps() == (s.predicted(), None)


def test_censored_cycles_only_raise_the_average():
    s = EMASchedule(engine=None, alpha=0.3)
    cycle(s, 0, trip=10)
    cycle(s, 10, end=14)                      # ended at 4 steps without a trip: no information
    assert s.predicted() == 10
    cycle(s, 14, end=30)                      # ran 16 steps without a trip: at least 16
    assert s.predicted() == pytest.approx(0.7 * 10 + 0.3 * 16)
    assert s.cycles == 3


def test_lengths_are_at_least_one_step():
    s = EMASchedule(engine=None, alpha=0.5)
    cycle(s, 5, trip=5)
    assert s.predicted() == 1
