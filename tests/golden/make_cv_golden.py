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
(H, F) inputs.

Usage (needs the reference checkout; the output is committed):
    python tests/golden/make_cv_golden.py /root/reference
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
    out_path = Path(__file__).with_name("cv_welford.npz")
    np.savez_compressed(out_path, **arrays)
    print(f"wrote {out_path} ({out_path.stat().st_size} bytes)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
