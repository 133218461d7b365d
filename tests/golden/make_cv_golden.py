"""Generates tests/golden/cv_welford.npz by running the REFERENCE's own
control-variate and Welford code (plugins/welford.py, plugins/cv_integrator.py,
plugins/metaintegrator.py of rgl-epfl/recursive_control_variates) on seeded
inputs.

Mitsuba / Dr.Jit are not installed, so the reference modules are imported
under a minimal stand-in: Dr.Jit float32 tensors become numpy float32 arrays
(`dr.select` -> np.where, `dr.clamp` -> np.clip, `dr.isnan/isinf`), the
integer sample count becomes a scalar whose `beta ** n` is the float32-rounded
power of the float32 beta, and every other Mitsuba symbol the modules touch
at import time is an inert placeholder.  Only the blend / statistics code
paths run; the nested tracer is replaced by a stub returning the recorded
(H, F) inputs (``render_twostates``) or recorded single-state images
(``render``), and logging the seed of every call.

Cases:
  * ``cases``: CVIntegrator / MetaIntegrator ``cv_ps`` blend sequences
    (plugins/cv_integrator.py:47-77, plugins/metaintegrator.py:57-130);
  * ``meta_cases``: MetaIntegrator sequences with the nested integrator's
    calls recorded: ``cv_pss`` (F = render(seed), H = the previous step's
    render(seed + 1), plugins/metaintegrator.py:87-91,117-119), the
    ``force_baseline`` returns of ``cv_pss`` and ``cv_ps``
    (plugins/metaintegrator.py:124-128) and the ``baseline`` method.

Usage (needs a checkout of the reference; the output is committed):
    python tests/golden/make_cv_golden.py <reference checkout>
or with the checkout in the environment variable RCV_REFERENCE.
"""
from __future__ import annotations

import sys
import types
import warnings
from pathlib import Path

import numpy as np

f32 = np.float32


class _Placeholder:
    """Inert stand-in: any attribute is another placeholder (capitalised
    names are classes so that the reference can subclass them), and calling
    one returns a placeholder."""

    def __init__(self, name="placeholder"):
        self._name = name

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        if name[:1].isupper():
            cls = type(name, (), {"__init__": lambda self, *a, **k: None})
            setattr(self, name, cls)
            return cls
        ph = _Placeholder(f"{self._name}.{name}")
        setattr(self, name, ph)
        return ph

    def __call__(self, *a, **k):
        return _Placeholder(self._name + "()")


class IntScalar:
    """Opaque scalar int tensor (mi.TensorXi) with float32 power semantics."""

    def __init__(self, v=0):
        self.v = int(v.v if isinstance(v, IntScalar) else v)

    def __gt__(self, o):
        return self.v > int(o)

    def __iadd__(self, o):
        self.v += int(o)
        return self

    def __int__(self):
        return self.v

    def __rpow__(self, base):
        return f32(float(f32(base)) ** self.v)


def make_fakes():
    dr = _Placeholder("drjit")
    dr.select = lambda c, a, b: np.where(c, a, b).astype(f32)
    dr.schedule = lambda *a, **k: None
    dr.make_opaque = lambda *a, **k: None
    dr.isnan = np.isnan
    dr.isinf = np.isinf
    dr.clamp = lambda x, lo, hi: np.clip(x, lo, hi).astype(f32)
    mi = _Placeholder("mitsuba")
    mi.TensorXf = lambda v=0.0: np.asarray(v, f32)
    mi.TensorXi = lambda v=0: IntScalar(v)

    class RBIntegrator:
        def __init__(self, props=None):
            pass

    mi.ad.integrators.common.RBIntegrator = RBIntegrator
    mi.load_dict = lambda d: _Placeholder("aov")
    return dr, mi


class Props(dict):
    def get(self, k, default=None):
        return super().get(k, default)


def import_reference(ref_root: Path):
    dr, mi = make_fakes()
    sys.modules["drjit"] = dr
    sys.modules["mitsuba"] = mi
    sys.path.insert(0, str(ref_root))
    import plugins.cv_integrator as cvi  # noqa: E402  (reference code)
    import plugins.metaintegrator as meta  # noqa: E402
    import plugins.twostatevolpath as tsv  # noqa: E402
    import plugins.welford as welford  # noqa: E402

    return cvi, meta, tsv, welford


def sequence(rng, steps, n, kind):
    """Seeded (H, F) sequences with the structure of consecutive iterates."""
    base = rng.uniform(0.0, 2.0, n).astype(f32)
    Hs, Fs = [], []
    prev = base
    for i in range(steps):
        drift = rng.normal(0.0, 0.02, n).astype(f32)
        cur = (prev + drift).astype(f32)
        noise_f = rng.normal(0.0, 0.3, n).astype(f32)
        noise_h = (noise_f * f32(0.9) + rng.normal(0.0, 0.1, n).astype(f32)).astype(f32)
        F = (cur + noise_f).astype(f32)
        H = (prev + noise_h).astype(f32)
        if kind == "edge":
            F[:4] = 0.0
            H[:4] = 0.0  # zero variance -> NaN weight -> 0
            F[4:8] = 1.5
            H[4:8] = 1.5  # constant pixels
            H[8:12] = F[8:12]  # H == F
            F[12:16] = f32(1e-30)  # tiny values
        Hs.append(H)
        Fs.append(F)
        prev = cur
    return np.stack(Hs), np.stack(Fs)


def run_cv(cls, tsv, Hs, Fs, props):
    inner = tsv.TwoStatePRBVolpathIntegrator(Props())
    feed = iter(zip(Hs, Fs))
    inner.render_twostates = lambda scene, sensor, seed, spp: next(feed)
    props = Props(props)
    props["integrator"] = inner
    integ = cls(props)
    outs = {"img": [], "w_s": [], "v_n": [], "var_x": [], "var_y": [], "cov": [], "mean_x": [], "mean_y": [], "n": []}
    for i in range(len(Hs)):
        img = integ.render(None, 0, i, 4)
        outs["img"].append(np.broadcast_to(np.asarray(img, f32), Hs[0].shape).copy())
        outs["w_s"].append(np.broadcast_to(np.asarray(integ.w_s, f32), Hs[0].shape).copy())
        outs["v_n"].append(np.broadcast_to(np.asarray(integ.v_n, f32), Hs[0].shape).copy())
        st = integ.stats
        for k in ("var_x", "var_y", "cov", "mean_x", "mean_y"):
            outs[k].append(np.broadcast_to(np.asarray(getattr(st, k), f32), Hs[0].shape).copy())
        outs["n"].append(int(st.n))
    return {k: np.asarray(v) for k, v in outs.items()}


class CallLog:
    """Nested-integrator stub: hands out recorded images in call order and
    logs (kind, seed) of every call (kind 0 = render_twostates, 1 = render)."""

    def __init__(self, twostate=(), single=()):
        self.twostate = iter(twostate)
        self.single = iter(single)
        self.calls = []

    def render_twostates(self, scene, sensor, seed, spp):
        self.calls.append((0, int(seed)))
        return next(self.twostate)

    def render(self, scene, sensor, seed, spp, develop=True, evaluate=True):
        self.calls.append((1, int(seed)))
        return next(self.single)


def run_meta(meta, tsv, props, steps, n, rng, seed0=5):
    """Drives the reference's MetaIntegrator with recorded nested renders.

    The nested renders form the sequences of consecutive iterates of
    ``sequence``: at step i the render with seed i of theta_i is F_i and the
    render with seed i + 1 of theta_i is H_{i+1} (the two-state pair of the
    next step)."""
    Hs, Fs = sequence(rng, steps + 1, n, "normal")
    method = props["method"]
    if method == "cv_ps":
        twostate = list(zip(Hs[:steps], Fs[:steps]))
        single = [(F + rng.normal(0.0, 0.05, n)).astype(f32) for F in Fs[:steps]]  # fresh baseline renders
    elif method == "cv_pss":
        twostate = []
        single = []
        for i in range(steps):
            single.append(Fs[i])
            single.append(Hs[i + 1])
    else:
        twostate = []
        single = [F.copy() for F in Fs[:steps]]
    inner = tsv.TwoStatePRBVolpathIntegrator(Props())
    log = CallLog(twostate, single)
    inner.render_twostates = log.render_twostates
    inner.render = log.render
    p = Props(props)
    p["integrator"] = inner
    integ = meta.MetaIntegrator(p)
    outs = {k: [] for k in ("out", "img", "w_s", "v_n", "var_x", "var_y", "cov", "n")}
    for i in range(steps):
        out = integ.render(None, 0, seed0 + i, 4)
        outs["out"].append(np.broadcast_to(np.asarray(out, f32), (n,)).copy())
        outs["img"].append(np.broadcast_to(np.asarray(integ.img, f32), (n,)).copy())
        if "cv" in method:
            outs["w_s"].append(np.broadcast_to(np.asarray(integ.w_s, f32), (n,)).copy())
            outs["v_n"].append(np.broadcast_to(np.asarray(integ.v_n, f32), (n,)).copy())
            for k in ("var_x", "var_y", "cov"):
                outs[k].append(np.broadcast_to(np.asarray(getattr(integ.stats, k), f32), (n,)).copy())
            outs["n"].append(int(integ.stats.n))
    res = {k: np.asarray(v) for k, v in outs.items() if len(v)}
    res["twostate_feed"] = np.asarray([np.stack(hf) for hf in twostate], f32).reshape(-1, 2, n)
    res["single_feed"] = np.asarray(single, f32).reshape(-1, n)
    res["calls"] = np.asarray(log.calls, np.int64).reshape(-1, 2)
    res["seed0"] = np.int64(seed0)
    return res


def main(ref_root: str):
    warnings.simplefilter("ignore")
    cvi, meta, tsv, welford = import_reference(Path(ref_root))
    rng = np.random.default_rng(20230801)
    cases = {}
    specs = [
        ("cv_default", cvi.CVIntegrator, {}, "normal"),
        ("cv_warmup3", cvi.CVIntegrator, {"warmup": 3}, "normal"),
        ("cv_betas", cvi.CVIntegrator, {"beta1": 0.5, "beta2": 0.9}, "normal"),
        ("cv_edge", cvi.CVIntegrator, {}, "edge"),
        ("meta_cv_ps", meta.MetaIntegrator, {"method": "cv_ps"}, "normal"),
        ("meta_pre_update", meta.MetaIntegrator, {"method": "cv_ps", "pre_update": True}, "normal"),
        ("meta_pre_update_edge", meta.MetaIntegrator, {"method": "cv_ps", "pre_update": True}, "edge"),
    ]
    for name, cls, props, kind in specs:
        Hs, Fs = sequence(rng, 12, 96, kind)
        out = run_cv(cls, tsv, Hs, Fs, props)
        cases[name] = (props, Hs, Fs, out)
    arrays = {}
    for name, (props, Hs, Fs, out) in cases.items():
        arrays[f"{name}/H"] = Hs
        arrays[f"{name}/F"] = Fs
        arrays[f"{name}/warmup"] = np.int32(props.get("warmup", 1))
        arrays[f"{name}/beta1"] = np.float32(props.get("beta1", 0.9))
        arrays[f"{name}/beta2"] = np.float32(props.get("beta2", 0.999))
        arrays[f"{name}/pre_update"] = np.int32(bool(props.get("pre_update", False)))
        for k, v in out.items():
            arrays[f"{name}/{k}"] = v
    # single-variable estimator
    xs = rng.normal(1.0, 0.5, (15, 64)).astype(f32)
    est = welford.WelfordVarianceEstimator(0.9, 0.999)
    means, variances, gets = [], [], []
    for x in xs:
        est.update(x)
        means.append(np.broadcast_to(np.asarray(est.mean, f32), x.shape).copy())
        variances.append(np.broadcast_to(np.asarray(est.var, f32), x.shape).copy())
        gets.append(np.asarray(est.get(), f32))
    arrays["welford1/x"] = xs
    arrays["welford1/mean"] = np.asarray(means)
    arrays["welford1/var"] = np.asarray(variances)
    arrays["welford1/get"] = np.asarray(gets)
    arrays["cases"] = np.array([c[0] for c in specs])
    # MetaIntegrator with its nested calls recorded (cv_pss, force_baseline)
    meta_specs = [
        ("meta_cv_pss", {"method": "cv_pss"}),
        ("meta_cv_pss_pre_update", {"method": "cv_pss", "pre_update": True}),
        ("meta_cv_pss_force", {"method": "cv_pss", "force_baseline": True}),
        ("meta_cv_ps_force", {"method": "cv_ps", "force_baseline": True}),
        ("meta_baseline", {"method": "baseline"}),
    ]
    for name, props in meta_specs:
        out = run_meta(meta, tsv, props, 10, 64, rng)
        arrays[f"{name}/method"] = np.array(props["method"])
        arrays[f"{name}/pre_update"] = np.int32(bool(props.get("pre_update", False)))
        arrays[f"{name}/force_baseline"] = np.int32(bool(props.get("force_baseline", False)))
        for k, v in out.items():
            arrays[f"{name}/{k}"] = v
    arrays["meta_cases"] = np.array([c[0] for c in meta_specs])
    out_path = Path(__file__).with_name("cv_welford.npz")
    np.savez_compressed(out_path, **arrays)
    print(f"wrote {out_path} ({out_path.stat().st_size} bytes)")


if __name__ == "__main__":
    import os

    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RCV_REFERENCE")
    if not root:
        sys.exit("usage: make_cv_golden.py <reference checkout>  (or set RCV_REFERENCE)")
    main(root)
