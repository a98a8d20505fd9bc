"""CPU checks of bench.py's host helpers: the committed ncu summaries carry the per-launch
figures the bench line reports (DRAM traffic of the dominant kernels, the batched pass's
instruction count per group), so the roofline fields are never silently null."""
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def test_profiles_carry_the_bench_figures():
    t_batch = bench.profile_traffic("cand_batch_10Mx1024_b8.md", "traffic_bytes_per_block")
    t_plain = bench.profile_traffic("cand_pass_10Mx1024_b8.md")
    ipg = bench.profile_number("cand_batch_10Mx1024_b8.md", "warp_instructions_per_group")
    # a 10M x 1024 8-bit launch reads about 491 MB of packets
    assert t_batch and 4.9e8 < t_batch < 6.0e8
    assert t_plain and 4.9e8 < t_plain < 6.0e8
    # about 22 instructions per group of four entries is the floor of the formulation
    assert ipg and 20 < ipg < 60
    assert bench.profile_number("cand_tc_2Mx1024_b4.md", "traffic_bytes_per_launch") > 2.5e9


def test_profile_number_missing_file_or_key():
    assert bench.profile_number("no_such_profile.md", "traffic_bytes_per_launch") is None
    assert bench.profile_number("cand_pass_10Mx1024_b8.md", "no_such_key") is None


def test_stale_profile_figures_are_not_reported(tmp_path, monkeypatch):
    # a summary whose digest names other kernel sources is not read
    name = "cand_pass_10Mx1024_b8.md"
    text = open(os.path.join(REPO, "profiles", name)).read()
    monkeypatch.setattr(bench, "REPO", str(tmp_path))
    os.makedirs(tmp_path / "profiles")
    os.makedirs(tmp_path / "acceles_gb300" / "csrc")
    for f in bench.PROFILE_SOURCES[name]:
        (tmp_path / "acceles_gb300" / "csrc" / f).write_text("// another build\n")
    (tmp_path / "profiles" / name).write_text(text)
    assert not bench.profile_current(name)
    assert bench.profile_traffic(name) is None


def test_reference_arm_loads_only_the_oracle():
    # the reference arm builds its matrix through the oracle: the engine library stays unloaded,
    # and its line carries the GPU arm's config keys and ms_per_step
    import json
    import subprocess
    code = (
        "import sys, json, io, contextlib; sys.argv=['bench.py','--impl','reference','--rows',"
        "'20000','--steps','2','--warmup','3','--cpu-step-queries','2']; import bench; "
        "buf=io.StringIO()\n"
        "with contextlib.redirect_stdout(buf): bench.main()\n"
        "maps=open('/proc/self/maps').read(); "
        "print(json.dumps({'line': json.loads(buf.getvalue()), "
        "'engine_loaded': 'libacceles' in maps, 'oracle_loaded': 'liboracle' in maps}))")
    r = subprocess.run([sys.executable, "-c", code], cwd=REPO, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert not d["engine_loaded"] and d["oracle_loaded"]
    line = d["line"]
    assert line["impl"] == "reference" and line["steps"] == 2 and line["ms_per_step"] > 0
    assert line["config"] == bench.headline_config(20000, line["config"]["nnz"], 1, 4096)


def test_every_workload_names_its_metric():
    """Each --workload leg prints a line with its own metric name (defined at module level)."""
    for name in ("METRIC", "SMALL_METRIC", "SERVE_METRIC"):
        assert isinstance(getattr(bench, name), str) and getattr(bench, name)
    import ast
    tree = ast.parse(open(bench.__file__).read())
    defined = {t.id for n in ast.walk(tree) if isinstance(n, ast.Assign) for t in n.targets
               if isinstance(t, ast.Name)}
    used = {n.id for n in ast.walk(tree) if isinstance(n, ast.Name) and n.id.endswith("METRIC")}
    assert used <= defined, used - defined
