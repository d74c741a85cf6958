"""Helpers shared by the GPU tests: device buffers (torch as plumbing),
synthetic workloads generated on the device, and the oracle run on the same
bytes."""
import os

import numpy as np

FIELDS = ("amplitudes", "chi2", "intime", "errors", "active_mask", "status", "iters")


class DeviceBatch:
    """Device buffers of one batch plus the mf_batch that points at them."""

    def __init__(self, mf, torch, n, stride=10, amp_stride=10, ctype=False):
        dev = "cuda"
        self.torch = torch
        self.n = n
        self.samples = torch.zeros((max(n, 1), stride), dtype=torch.float64, device=dev)
        self.pederr = torch.zeros(max(n, 1), dtype=torch.float64, device=dev)
        self.ctype = torch.zeros(max(n, 1), dtype=torch.uint8, device=dev) if ctype else None
        self.out = {
            "amplitudes": torch.zeros((max(n, 1), amp_stride), dtype=torch.float64, device=dev),
            "chi2": torch.zeros(max(n, 1), dtype=torch.float64, device=dev),
            "intime": torch.zeros(max(n, 1), dtype=torch.float64, device=dev),
            "errors": torch.zeros(max(n, 1), dtype=torch.float64, device=dev),
            "active_mask": torch.zeros(max(n, 1), dtype=torch.int16, device=dev),
            "status": torch.zeros(max(n, 1), dtype=torch.uint8, device=dev),
            "iters": torch.zeros(max(n, 1), dtype=torch.int32, device=dev),
        }
        self.batch = mf.Engine._batch(
            n, stride, amp_stride, self.samples.data_ptr(), self.pederr.data_ptr(),
            self.ctype.data_ptr() if ctype else None, self.out["amplitudes"].data_ptr(),
            self.out["chi2"].data_ptr(), self.out["intime"].data_ptr(), self.out["errors"].data_ptr(),
            self.out["active_mask"].data_ptr(), self.out["status"].data_ptr(), self.out["iters"].data_ptr())

    def generate(self, mf, params, first=0):
        mf.synth_generate_device(params, first, self.n, self.samples.data_ptr(), self.pederr.data_ptr(),
                                 self.ctype.data_ptr() if self.ctype is not None else None,
                                 stride=self.samples.shape[1])
        self.torch.cuda.synchronize()

    def inputs_host(self):
        d = {"samples": self.samples[: self.n].cpu().numpy(), "pederr": self.pederr[: self.n].cpu().numpy()}
        d["ctype"] = self.ctype[: self.n].cpu().numpy() if self.ctype is not None else np.zeros(self.n, np.uint8)
        return d

    def outputs_host(self):
        self.torch.cuda.synchronize()
        o = {k: v[: self.n].cpu().numpy() for k, v in self.out.items()}
        o["active_mask"] = o["active_mask"].view(np.uint16)
        return o


def oracle_fit_sets(mf, oracle, engine, inputs, **kw):
    """Runs the oracle per condition set on host inputs, scattering into full-size outputs."""
    n = inputs["samples"].shape[0]
    res = {"amplitudes": np.zeros((n, 10)), "chi2": np.zeros(n), "active_mask": np.zeros(n, np.uint16),
           "status": np.zeros(n, np.uint8), "iters": np.zeros((n, 3), np.int32), "errors": np.zeros(n)}
    if kw.get("count_flops"):
        res["flops"] = np.zeros(n)
    for t, cond in engine.conditions.items():
        sel = np.nonzero(inputs["ctype"] == t)[0]
        if sel.size == 0:
            continue
        P, R, bxs, F = mf.conditions_arrays(cond)
        o = oracle.fit_batch(inputs["samples"][sel], inputs["pederr"][sel], P, R, bxs, fullpulsecov=F, **kw)
        K = P.shape[1]
        res["amplitudes"][sel, :K] = o["amplitudes"]
        for k in ("chi2", "active_mask", "status", "iters", "errors"):
            res[k][sel] = o[k]
        if kw.get("count_flops"):
            res["flops"][sel] = o["flops"]
    return res


def pack_iters(it3):
    it3 = np.asarray(it3, dtype=np.int64)
    return (np.minimum(it3[:, 0], 255) | (np.minimum(it3[:, 1], 4095) << 8) |
            (np.minimum(it3[:, 2], 4095) << 20)).astype(np.int32)


def assert_bitwise(gpu, ref, fields=("amplitudes", "chi2", "active_mask", "status"), iters=True, sel=None):
    for k in fields:
        g = gpu[k] if sel is None else gpu[k][sel]
        r = ref[k] if sel is None else ref[k][sel]
        if k == "amplitudes":
            g = g[:, : r.shape[1]]
        if g.dtype.kind == "f":
            same = (g == r) | (np.isnan(g) & np.isnan(r))
        else:
            same = g == r
        if not same.all():
            bad = np.argwhere(~same)[:5]
            raise AssertionError(f"{k}: {(~same).sum()} mismatches, first {bad.tolist()}: "
                                 f"gpu {g[tuple(bad[0])]!r} oracle {r[tuple(bad[0])]!r}")
    if iters:
        g = gpu["iters"] if sel is None else gpu["iters"][sel]
        r = pack_iters(ref["iters"] if sel is None else ref["iters"][sel])
        assert np.array_equal(g, r), "iteration counters differ"


COMMITTED_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_data")


def reference_data_dir():
    """The reference tree's data/ directory (the tree the oracle recipe
    compiles from) where it exists, else the two data files committed under
    tests/golden/reference_data/ (made by tests/golden/make_reference_data.py)."""
    from oracle import build_oracle

    d = os.path.join(build_oracle.REFERENCE_ROOT, "data")
    return d if os.path.isdir(d) else COMMITTED_DATA


def replay_data_dir():
    """The directory of the reference's data files for the GPU replay tests:
    MULTIFIT_REPLAY_DATA where the user names one, else the committed copies
    under tests/golden/reference_data/."""
    return os.environ.get("MULTIFIT_REPLAY_DATA") or COMMITTED_DATA
