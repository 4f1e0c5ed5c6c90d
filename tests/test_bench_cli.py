"""bench.py's command line, the interface the benchmark runs through: the
documented flags parse, and the workload configurations it reports are
complete.  No GPU: only the parser and the configuration tables run."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_help_lists_the_documented_flags():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True,
                         text=True, cwd=ROOT, timeout=120)
    assert out.returncode == 0, out.stderr
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--no-cpu-baseline", "--no-reference-cuda",
                 "--no-part", "--cell-tiles", "--blend-shape", "--tile-schedule", "--stage-entries"):
        assert flag in out.stdout, flag


def test_workload_configs_name_their_sizes():
    sys.path.insert(0, ROOT)
    import bench
    c = bench._workload_config("sq500k_16x800x600")
    assert c["workload"] == "sq500k_16x800x600"
    assert (c["surfels"], c["views"], c["height"], c["width"]) == (500_000, 16, 600, 800)
