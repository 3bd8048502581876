"""bench.py host logic that needs no GPU: a failing secondary measurement is recorded in
the JSON line instead of ending the run."""

import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_secondary_measurement_failure_is_recorded():
    bench = _bench()

    def boom(x):
        raise RuntimeError(f"no device {x}")

    assert bench.measured(lambda a, b: a + b, 2, 3) == 5
    assert bench.measured(boom, 7) == {"error": "RuntimeError: no device 7"}
