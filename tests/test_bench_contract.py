"""bench.py's JSON contract, checked on the CPU through its reference arm
(the reference's CPU algorithm: the oracle on the host cores)."""
import json
import pathlib
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2", "--warmup",
                        "1", "--workload", "config0_f64"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key, typ in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                     ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                     ("dtype", str), ("data", str), ("config", dict), ("e2e", dict), ("cpu_baseline", dict)):
        assert isinstance(d[key], typ), key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["unit"] == "cell-steps/s" and d["higher_is_better"] is True
    assert d["vs_baseline"] is None and d["scaling"] in ("weak", "strong")
    assert d["config"]["workload"] == "config0_f64"
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]


def test_reference_arm_under_torchrun_prints_once():
    """Launched like the multi-GPU runs (torchrun, 2 ranks on 127.0.0.1):
    rank 0 prints the one line, the other rank exits 0 without work."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
                        "--impl", "reference", "--steps", "1", "--warmup", "0", "--workload", "config0_f64"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["impl"] == "reference"


def test_reference_arm_loads_no_gpu_library_and_prints_the_same_config():
    """The reference arm makes its inputs with libgbf_inputs.so and never maps
    libgbflow; its `config` equals the one the GPU arm builds for the same
    workload from libgbflow's generator."""
    code = (
        "import json, sys, types; sys.path.insert(0, %r); import bench, __graft_entry__ as ge\n"
        "a = types.SimpleNamespace(workload='config4_split', cube=0, members=3, steps=1, warmup=0)\n"
        "out = bench.run_reference(a, 0, 1)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'config': out['config'], 'gbflow': 'libgbflow' in maps,\n"
        "                  'inputs': 'libgbf_inputs' in maps, 'oracle': 'libgbf_oracle' in maps}))\n" % str(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert not d["gbflow"] and d["inputs"] and d["oracle"]
    import __graft_entry__ as ge
    sys.path.insert(0, str(ROOT))
    import bench
    pkg = ge.load_package()
    W = bench.Workload(pkg, pkg.load_library(), "config4_split", 0, 0, 1, 3)
    assert W.config() == d["config"]


def test_dropin_split_workload_names_its_form_and_grid():
    """config1_dropinsplit: config 1's media-table grid through the defines.h
    calls in split mode; the drop-in forms refuse other configurations."""
    import pytest
    import __graft_entry__ as ge
    sys.path.insert(0, str(ROOT))
    import bench
    pkg = ge.load_package()
    lib = pkg.load_library()
    W = bench.Workload(pkg, lib, "config1_dropinsplit", 16, 0, 1)
    fused = bench.Workload(pkg, lib, "config1_dropin", 16, 0, 1)
    assert bench.DROPIN_MODES == {"dropin": 1, "dropinsplit": 2}
    c, cf = W.config(), fused.config()
    assert c["workload"] == "config1_dropinsplit" and c["desc"] == cf["desc"] and c["cells"] == 16 ** 3
    assert "split mode" in c["form"] and "fused mode" in cf["form"]
    assert W.members[0].media is not None and W.members[0].K is None
    assert bench.ALGO_BYTES_DROPIN["split_step"] == (52.0, "interior")
    with pytest.raises(SystemExit):
        bench.Workload(pkg, lib, "config2_dropinsplit", 0, 0, 1)
