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


def test_reference_config_carries_every_field():
    """The reference's own SimulationConfig built from the bench workload's has the same
    value in every field the reference defines (it is what the reference arm times)."""
    import dataclasses
    import sys

    import pytest

    from fixtures import reference_src

    src = reference_src()
    if not src:
        pytest.skip("reference sources not present")
    sys.path.insert(0, src)
    bench = _bench()
    from pyalbsim_gb300.workloads import large

    ours = large()
    ref = bench._reference_config(ours)
    assert type(ref).__module__.startswith("alb_sim.")

    def compare(a, b):
        if dataclasses.is_dataclass(b):
            for f in dataclasses.fields(b):
                compare(getattr(a, f.name), getattr(b, f.name))
        elif isinstance(b, tuple):
            assert len(a) == len(b)
            for x, y in zip(a, b):
                compare(x, y)
        else:
            assert a == b

    compare(ours, ref)
    with pytest.raises(ValueError):  # an extension field set has no counterpart in the reference
        bench._reference_config(large(hg=0.9))


def test_cpu_model_is_reported():
    assert isinstance(_bench().cpu_model(), str) and _bench().cpu_model()


def test_gather_issue_roofline_arithmetic():
    """The issue roofline of the scatter gather: instructions per query x queries over the
    kernel time, against SMs x 4 schedulers x the clock."""
    bench = _bench()
    r = bench.gather_issue_roofline(1_000_000, 10.0, sms_mhz=(152, 2070.0))
    assert r["peak"] == 152 * 4 * 2070.0e6
    assert abs(r["achieved"] - bench.INST_PER_SCATTER_QUERY * 1e6 / 0.01) < 1e-3
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-15
    assert bench.gather_issue_roofline(5, 0.0, sms_mhz=(152, 2070.0))["achieved"] == 0.0
