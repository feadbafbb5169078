"""bench.py's host side without a GPU: the timed CPU baseline loop is the
oracle's step, the clock record is read the way the timing rules need
(median SM clock under load, maximum clock, throttle reasons seen), and the
blocking error behind the ZPE error bars recovers the known standard error
of a correlated series."""
import numpy as np

import bench
import oracle


def test_timed_cpu_step_is_the_oracle_step():
    p, m = oracle.h2o_config()
    x0 = bench.start_structures(300, 5)
    pes = lambda c: oracle.pes_h2o_lm(c, p)  # noqa: E731
    whole = oracle.OracleDMC(x0, m, bench.DT, pes, bench._NumpyNoise(1)).run(7)
    timed = oracle.OracleDMC(x0, m, bench.DT, pes, bench._NumpyNoise(1)).run(3)
    for _ in range(4):
        bench._single_step(timed)
    assert np.array_equal(timed.x, whole.x)
    assert timed.vref == whole.vref


def test_cpu_reference_rate_runs_at_least_the_steps_asked():
    rate, secs, k = bench.cpu_reference_rate(200, 3, 1)
    assert k == 3 and secs > 0 and rate > 0
    rate, secs, k = bench.cpu_reference_rate(200, 1, 1, min_s=0.05, max_steps=10 ** 6)
    assert secs >= 0.05 and k >= 1


def test_clock_record_summary(tmp_path):
    rows = ["0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
            "0, 2055, 2070, 1380.0, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 2070, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
            "garbage line"]
    f = tmp_path / "clocks.csv"
    f.write_text("\n".join(rows) + "\n")
    c = bench.ClockSampler(0)
    c.proc = object()  # as if nvidia-smi had been started
    with open(f) as c.f:
        s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.ClockSampler(0).summary()["reasons"] == ["nvidia-smi unavailable"]


def test_blocking_error_of_a_correlated_series():
    # AR(1), phi = 0.9: the standard error of the mean is sqrt(var * tau / n) with
    # var = 1 / (1 - phi^2) and tau = (1 + phi) / (1 - phi) = 19, 4.4x the naive iid value
    import pyvibdmc_gb300 as pg
    phi, n = 0.9, 200000
    e = np.random.default_rng(3).standard_normal(n)
    x = np.empty(n)
    x[0] = e[0]
    for t in range(1, n):
        x[t] = phi * x[t - 1] + e[t]
    mean, err = pg.blocking_error(x, 20)
    true = np.sqrt(1 / (1 - phi ** 2) * (1 + phi) / (1 - phi) / n)
    assert abs(mean) < 5 * true
    assert 0.5 * true < err < 1.5 * true
    assert err > 2.5 * x.std() / np.sqrt(n)
    assert pg.blocking_error([1.0, 2.0, 3.0])[0] == 2.0  # short series: two blocks
