"""The surrogate gate's calibration rule, on the CPU (torch tensors; no GPU).

Surrogate.threshold(g, e, bound) returns the largest gate score up to which
every calibration state has error e <= bound: the network serves a state
when its score is at or below the threshold, so a threshold must stop
before the first state over the bound, and a state tied with that one must
not be served either.
"""
import pytest

torch = pytest.importorskip("torch")

from create_rate_subs_gb300.surrogate import Surrogate


def test_threshold_stops_before_the_first_state_over_the_bound():
    g = torch.tensor([0.1, 0.5, 0.3, 0.9, 0.7])
    e = torch.tensor([0.0, 0.0, 0.0, 1.0, 0.0])
    assert Surrogate.threshold(g, e, 0.5) == pytest.approx(0.7)


def test_threshold_when_the_best_scored_state_is_over():
    g = torch.tensor([0.1, 0.5, 0.3])
    e = torch.tensor([1.0, 0.0, 0.0])
    assert Surrogate.threshold(g, e, 0.5) == float("-inf")


def test_threshold_excludes_ties_with_the_first_bad_state():
    g = torch.tensor([0.1, 0.3, 0.3])
    e = torch.tensor([0.0, 0.0, 1.0])
    assert Surrogate.threshold(g, e, 0.5) == pytest.approx(0.1)


def test_threshold_serves_everything_when_nothing_is_over():
    g = torch.tensor([0.1, 0.3, 0.3])
    assert Surrogate.threshold(g, torch.zeros(3), 0.5) == pytest.approx(0.3)


def test_threshold_rule_holds_on_random_scores():
    """Every state at or below the threshold is within the bound, and the
    next score up belongs to a state over it."""
    gen = torch.Generator().manual_seed(0)
    g = torch.rand(10000, generator=gen)
    e = (g + 0.3 * torch.rand(10000, generator=gen)) ** 2
    tau = Surrogate.threshold(g, e, 0.2)
    served = g <= tau
    assert bool((e[served] <= 0.2).all())
    g_next = g[~served].min()  # the first score the gate sends back
    assert bool(((g == g_next) & (e > 0.2)).any())
