"""CPU: the reference's own drivers, unchanged, driving this engine (ES_ENGINE=es_gb300).

The drop-in claim is that harness/run_k.py, harness/run_k_masks.py and the CLI line that
harness/replay_release.py builds run against es_gb300 with no edit.  Here those files are
imported from the reference checkout as they are, and the engine's device half is replaced by
the oracle-backed fake of tests/fake_device.py, so what runs is the reference's own block loop,
checkpoint/resume logic and CLI over es_gb300's GpuSieve surface:

* harness/run_k.py main(): g(k) equals the b-file for every k <= 60 (harness/gate_driver.py's
  check), and the gate's resume test -- a ``--max-blocks 2 --ckpt-every 0`` first pass, then a
  resumed pass -- reaches the same g with ``restarts`` > 0;
* harness/run_k.py run() stopped in the middle of a block and resumed from its checkpoint gives
  the same block audit as an uninterrupted run (the ``unit_done`` / ``idx_done`` arithmetic);
* harness/run_k_masks.py main(): FOUND with the b-file value, ``--max-launches`` pauses mid-block
  and a resume completes, the checkpoint records the engine's ``mask_mode``, and ``--ban`` goes
  through the engine's ``plan_wheel``;
* harness/replay_release.py command(): the argv it builds for a recorded frontier wheel parses
  and runs against es_gb300.main, whose JSON line carries the recorded wheel's modulus and
  residues per block.

The reference checkout is found through ES_REFERENCE_ROOT or as the ``reference`` directory
beside this repository; without it these tests are skipped (it never travels to a GPU host).
"""
import importlib.util
import io
import json
import os
import sys
from contextlib import redirect_stdout

import pytest

from fake_device import install

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_root():
    for cand in (os.environ.get("ES_REFERENCE_ROOT"), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.isfile(os.path.join(cand, "harness", "run_k.py")):
            return cand
    return None


REF = _reference_root()
pytestmark = pytest.mark.skipif(REF is None, reason="reference checkout not present")


@pytest.fixture
def driver(monkeypatch):
    """Import a reference harness module as it is, with ES_ENGINE=es_gb300; sys.path and the
    module table are restored afterwards."""
    saved_path = list(sys.path)
    saved_mods = set(sys.modules)
    monkeypatch.setenv("ES_ENGINE", "es_gb300")

    def load(name):
        spec = importlib.util.spec_from_file_location(f"_ref_{name}", os.path.join(REF, "harness", f"{name}.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod
    yield load
    sys.path[:] = saved_path
    for m in set(sys.modules) - saved_mods:
        if m.startswith("_ref_") or m == "erdos_ref":
            del sys.modules[m]


def _cli(mod, monkeypatch, argv):
    """Run a reference CLI's main() with argv; returns the last JSON line it printed."""
    monkeypatch.setattr(sys, "argv", [mod.__file__] + [str(a) for a in argv])
    buf = io.StringIO()
    with redirect_stdout(buf):
        mod.main()
    lines = [ln for ln in buf.getvalue().splitlines() if ln.startswith("{")]
    return json.loads(lines[-1])


def test_run_k_gate_matches_bfile(driver, monkeypatch, tmp_path, bfile):
    """harness/gate_driver.py's check through run_k.py's CLI: FOUND g(k) = b-file, k = 1..60."""
    run_k = driver("run_k")
    install(monkeypatch)
    for k in range(1, 61):
        res = _cli(run_k, monkeypatch, [k, "--tag", "gate", "--ckpt-dir", tmp_path, "--log-every", "1e9",
                                        "--ckpt-every", "1e9", "--no-resume"])
        assert res["status"] == "FOUND" and int(res["g"]) == bfile[k], (k, res)
        assert res["engine_module"] == "es_gb300" and res["matches_bfile"] is True


@pytest.mark.parametrize("k", [30, 57, 117])
def test_run_k_gate_resume(driver, monkeypatch, tmp_path, bfile, k):
    """harness/gate_driver.py's resume test: stop after 2 blocks with a checkpoint, resume."""
    run_k = driver("run_k")
    install(monkeypatch)
    common = ["--tag", f"resume{k}", "--ckpt-dir", tmp_path, "--log-every", "1e9"]
    r1 = _cli(run_k, monkeypatch, [k] + common + ["--no-resume", "--max-blocks", "2", "--ckpt-every", "0"])
    ck = json.load(open(tmp_path / f"k{k}_resume{k}.json"))
    assert r1["status"] == "EXHAUSTED_BLOCKS" and ck["t"] == 2
    r2 = _cli(run_k, monkeypatch, [k] + common + ["--ckpt-every", "1e9"])
    assert r2["status"] == "FOUND" and int(r2["g"]) == bfile[k]
    assert r2["restarts"] > 0 and r2["block"] >= 2


def test_run_k_mid_block_resume_same_audit(driver, monkeypatch, tmp_path, bfile):
    """run_k.run() stopped by its timeout in the middle of a block (after 5 of the block's
    launches), then resumed from the checkpoint: same g and the same per-block audit records
    (counts and survivor hashes) as one uninterrupted run."""
    run_k = driver("run_k")
    made = install(monkeypatch)
    k, tun = 60, {"chunk_log2": 7}   # 9 launches per block
    full = run_k.run(k, str(tmp_path / "full.json"), tun, None, None, None, 1e9, 1e9, 0, False)
    assert full["status"] == "FOUND" and int(full["g"]) == bfile[k]

    real_time = run_k.time.time

    class Clock:   # wall time jumps past the timeout once the fake has run 5 launches
        @staticmethod
        def time():
            return real_time() + (1e6 if made and made[-1].launches >= 5 else 0.0)

        def __getattr__(self, name):
            return getattr(run_k.time, name)
    monkeypatch.setattr(run_k, "time", Clock())
    made.clear()
    ck = str(tmp_path / "part.json")
    part = run_k.run(k, ck, tun, None, None, 10.0, 1e9, 1e9, 0, False)
    state = json.load(open(ck))
    assert part["status"] == "TIMEOUT" and 0 < state["unit_done"] < part["units_total"]
    assert state["idx_done"] == state["unit_done"] * made[-1].r0
    monkeypatch.setattr(run_k, "time", sys.modules["time"])
    resumed = run_k.run(k, ck, tun, None, None, None, 1e9, 1e9, 0, True)
    assert resumed["status"] == "FOUND" and resumed["g"] == full["g"] and resumed["restarts"] == 1
    assert resumed["block_audit"] == full["block_audit"]


def test_run_k_masks_found_pause_resume_and_mask_mode(driver, monkeypatch, tmp_path, bfile):
    """harness/run_k_masks.py: FOUND = b-file; --max-launches pauses in the middle of a block and
    the resumed run completes; the checkpoint records the engine's mask_mode."""
    masks = driver("run_k_masks")
    install(monkeypatch)
    k = 70
    base = [k, "--ckpt-dir", tmp_path, "--log-every", "1e9", "--tune", json.dumps({"chunk_log2": 7})]
    res = _cli(masks, monkeypatch, base + ["--tag", "whole", "--no-resume", "--ckpt-every", "1e9"])
    assert res["status"] == "FOUND" and int(res["g"]) == bfile[k]
    r1 = _cli(masks, monkeypatch, base + ["--tag", "paused", "--no-resume", "--ckpt-every", "0",
                                          "--max-launches", "3"])
    assert r1["status"] == "PAUSED" and 0 < r1["unit_done"] < r1["units_total"]
    state = json.load(open(tmp_path / f"k{k}_paused.json"))
    assert state["mask_mode"] in ("wordmask-gb300", "pair-gb300", "smem-gb300", "smem-pair-gb300", "auto-gb300",
                                  "scalar-gb300")
    r2 = _cli(masks, monkeypatch, base + ["--tag", "paused", "--ckpt-every", "1e9"])
    assert r2["status"] == "FOUND" and r2["g"] == res["g"] and r2["restarts"] == 1
    assert r2["block_audit"] == res["block_audit"]


def test_run_k_ban_uses_engine_planner(driver, monkeypatch, tmp_path, bfile):
    """--ban rebuilds the wheel through the engine module's plan_wheel and TUNABLES."""
    run_k = driver("run_k")
    install(monkeypatch)
    res = _cli(run_k, monkeypatch, [50, "--ban", "3", "--tag", "ban", "--ckpt-dir", tmp_path, "--log-every", "1e9",
                                    "--ckpt-every", "1e9", "--no-resume"])
    assert res["status"] == "FOUND" and int(res["g"]) == bfile[50]
    assert 3 not in [p for p, _ in res["plan"]["wheel"]]


@pytest.mark.parametrize("k,role", [(378, "primary"), (390, "confirmation")])
def test_replay_release_command_runs_engine_cli(driver, monkeypatch, capsys, k, role):
    """The argv harness/replay_release.py builds for a recorded wheel, pointed at es_gb300.py
    instead of the archived engine file, parses and runs through es_gb300.main; the search is
    stubbed (a whole frontier block is hours of GPU time), the plan is real."""
    import es_gb300
    rel = driver("replay_release")
    argv = rel.command(k, role)
    assert argv[1].endswith("gpu_sieve_v9.py")
    runs = {t["k"]: t for t in json.load(open(os.path.join(REF, "evidence", "through400", "runs.json")))["terms"]}
    rec = runs[k][role]
    seen = {}

    class StubSieve:
        def __init__(self, plan):
            seen["plan"] = plan

        def search(self, max_blocks, log=None):
            seen["max_blocks"] = max_blocks
            return {"k": k, "status": "EXHAUSTED_BLOCKS", "blocks": max_blocks, "residues_checked": 0, "wall": 0.0}
    monkeypatch.setattr(es_gb300, "GpuSieve", StubSieve)
    monkeypatch.setattr(es_gb300, "free_vram_mib", lambda: None)
    es_gb300.main(argv[2:])
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert seen["max_blocks"] == rec["block"] + 1
    assert line["plan"]["wheel"] == [list(w) for w in rec["wheel"]]
    assert int(line["plan"]["N"]) == int(rec["N"])
    assert int(line["plan"]["residues_per_block"]) == int(rec["residues_per_block"])
