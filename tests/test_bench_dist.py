"""The multi-rank logic of bench.py on CPU: two gloo ranks (torch.distributed,
world size 2) run the replicas path -- each fits its own contiguous shard of
the seeded channel stream with no data-path collective -- and the timing
reduction is a max over ranks. The shards' fits (the oracle, on the host)
concatenate to the single-process fit of the whole stream, and the CPU
reference arm runs on rank 0 only."""
import importlib.util
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    bench = load_bench()
    import argparse

    import torch.distributed as dist

    args = argparse.Namespace(impl="ours")
    w, r, _ = bench.dist_setup(args)
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    mf = bench.load_pkg()
    import oracle

    per = 300
    first, count = bench.shard_range(r, per)
    p = mf.WORKLOADS["ecal-10k-pu0.5"]()
    d = mf.synth_generate_host(p, first, count, with_truth=False)
    P, R, bxs, _ = mf.conditions_arrays(mf.synth_conditions(mf.SYNTH_ECAL)[0])
    o = oracle.fit_batch(d["samples"], d["pederr"], P, R, bxs, nthreads=1)
    bench.barrier(w)
    mx = bench.max_over_ranks(10.0 + r, w)
    np.savez(os.path.join(out_dir, f"rank{r}.npz"), amplitudes=o["amplitudes"], chi2=o["chi2"], first=first,
             mx=mx)
    # the reference arm: rank 0 prints one JSON line, the other ranks return without work
    ref_args = argparse.Namespace(impl="reference", form="fp64", workload="ecal-10k-pu0.5", max_iter=10, start=0,
                                  steps=1, warmup=0, cpu_seconds=0.05)
    res = bench.run_reference(ref_args, w, r)
    with open(os.path.join(out_dir, f"ref{r}.json"), "w") as f:
        json.dump(res, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_fit_disjoint_shards(mf, tmp_path):
    import torch.multiprocessing as tmp

    world = 2
    tmp.spawn(rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world, join=True)
    parts = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]
    assert [int(q["first"]) for q in parts] == [0, 300]
    assert all(float(q["mx"]) == 11.0 for q in parts)
    import oracle

    d = mf.synth_generate_host(mf.WORKLOADS["ecal-10k-pu0.5"](), 0, 600, with_truth=False)
    P, R, bxs, _ = mf.conditions_arrays(mf.synth_conditions(mf.SYNTH_ECAL)[0])
    whole = oracle.fit_batch(d["samples"], d["pederr"], P, R, bxs, nthreads=1)
    assert np.array_equal(np.concatenate([q["amplitudes"] for q in parts]), whole["amplitudes"])
    assert np.array_equal(np.concatenate([q["chi2"] for q in parts]), whole["chi2"])
    refs = [json.load(open(tmp_path / f"ref{r}.json")) for r in range(world)]
    assert refs[1] is None
    assert refs[0]["impl"] == "reference" and refs[0]["n_gpus"] == 2 and refs[0]["value"] > 0
    assert refs[0]["e2e"]["h2d_bytes_per_step"] == 0
