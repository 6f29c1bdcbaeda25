"""The chosen method's Newton settings (intpointsfem_gb300.use_chosen_newton)
as host logic: which setters it calls with which values, on a recording
stand-in for the struct matrix (no device needed)."""
import intpointsfem_gb300 as ip


class _Recorder:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def rec(*a, **k):
            self.calls.append((name, a, k))
        return rec


def test_use_chosen_newton_applies_the_chosen_settings():
    r = _Recorder()
    ip.use_chosen_newton(r)
    calls = {name: (a, k) for name, a, k in r.calls}
    assert set(calls) == {"set_inner_tolerance", "set_newton_predictor", "set_consistent_tangent"}
    assert calls["set_inner_tolerance"] == ((), ip.CHOSEN_INNER)
    assert ip.CHOSEN_INNER == dict(mode=1, gamma=0.9, alpha=2.0, eta_min=1e-4, eta_max=0.3)
    assert calls["set_newton_predictor"] == ((True,), {})
    assert calls["set_consistent_tangent"] == ((True,), {})
    assert ip.CHOSEN_CG_RTOL == 3e-2
