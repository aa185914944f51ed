"""Restatement of the reference Logger's latency statistics, for tests only.

core/logger.hpp:197-243 (analyse): latencies of a query class are sorted; the
median is element n / 2 and the 99th percentile element floor(n * 0.99).
core/logger.hpp:254-305 (print_cdf): the CDF is sampled at 25 rates -- 0.01,
then 0.05 .. 0.95 by 0.05, then 0.96 .. 1.00 by 0.01 -- each at element
floor(n * rate), clamped to the last element.  This is test infrastructure:
the library computes the same statistics itself (wk_server_get_stats,
wk_server_latency_cdf)."""


def cdf_rates():
    rates = [0.01] + [0.05 * i for i in range(1, 20)] + [0.95 + 0.01 * i for i in range(1, 6)]
    assert len(rates) == 25
    return rates


def at_rate(latencies, rate):
    v = sorted(latencies)
    if not v:
        return 0.0
    i = int(len(v) * rate)
    return v[min(i, len(v) - 1)]


def cdf(latencies):
    return [at_rate(latencies, r) for r in cdf_rates()]
