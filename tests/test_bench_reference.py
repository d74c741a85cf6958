"""bench.py's reference arm on CPU: it times the reference's CPU path (the
oracle port) on inputs from the oracle's own generator, never loads the
engine library, and prints the same `config` the GPU arm prints for the same
command line, with one-thread and multifit_cpu-setting legs beside it."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
import importlib.util, json, sys, argparse
sys.path.insert(0, {root!r})
spec = importlib.util.spec_from_file_location("bench_ref", {bench!r})
b = importlib.util.module_from_spec(spec); spec.loader.exec_module(b)
args = argparse.Namespace(impl="reference", form={form!r}, workload="ecal-10k-pu0.5", max_iter=10, start=0,
                          steps=2, warmup=1, cpu_seconds=0.2, channels=0, ref_step_cap_s=8.0)
out = b.run_reference(args, 1, 0)
maps = open("/proc/self/maps").read()
print("RESULT " + json.dumps({{"line": out, "engine_mapped": "libmultifit_gb300" in maps,
                              "engine_module": "multifit_gb300" in sys.modules,
                              "config_ours": b.workload_config(args, "ecal-10k-pu0.5", 10000, 1)}}))
"""


def run(form):
    code = PROG.format(root=ROOT, bench=os.path.join(ROOT, "bench.py"), form=form)
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-3000:]
    line = [ln for ln in res.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    return json.loads(line[len("RESULT "):])


def test_reference_arm_loads_no_engine_and_matches_config():
    r = run("warm")
    line = r["line"]
    assert not r["engine_mapped"] and not r["engine_module"]
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"] == r["config_ours"]
    assert line["config"]["channels_per_step"] == 10000
    assert "KKT" in line["config"]["fit"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"]
    assert cb["one_thread"]["threads"] == 1 and cb["one_thread"]["value"] > 0
    assert cb["multifit_cpu_settings"]["all_threads"]["value"] > 0
    assert cb["multifit_cpu_settings"]["one_thread"]["threads"] == 1
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "all 10000 channels" in cb["sample"]


def test_reference_arm_fp64_form_uses_the_command_line_fit():
    line = run("fp64")["line"]
    assert "multifit_cpu literal" in line["config"]["fit"]
