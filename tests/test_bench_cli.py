"""bench.py's command line without a GPU: it parses, and it offers the
flags the benchmark contract and the committed profile commands use."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_help_lists_contract_flags():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], cwd=ROOT,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--exec", "--arith", "--no-cpu-baseline",
                 "--sections", "--batch-mode", "--batch-mats"):
        assert flag in out.stdout, flag


def test_profile_commands_use_known_flags():
    """Every bench.py flag named in a profiles/ command exists."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], cwd=ROOT,
                         capture_output=True, text=True, timeout=300).stdout
    prof = os.path.join(ROOT, "profiles")
    for name in sorted(os.listdir(prof)):
        if not name.endswith(".md"):
            continue
        for line in open(os.path.join(prof, name)):
            if "bench.py" not in line:
                continue
            words = line.replace("\\", " ").split()
            i = words.index("bench.py") if "bench.py" in words else -1
            for w in words[i + 1:]:
                if w.startswith("--"):
                    assert w in out, f"{name}: {w}"
                if w in ("&&", ">", "2>&1"):
                    break


def test_profile_commands_run_committed_files_only():
    """The commands in profiles/ name no working-directory scripts."""
    prof = os.path.join(ROOT, "profiles")
    for name in sorted(os.listdir(prof)):
        if name.endswith(".md"):
            text = open(os.path.join(prof, name)).read()
            assert "_work/" not in text, name
