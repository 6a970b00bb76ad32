"""bench.py --impl reference: the JSON line the reference arm prints, timing the
reference binary (oracle/_ref/main) where it exists and runs, else the oracle
port, on a small sample so the test stays quick."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _Args:
    gpus, steps, warmup, config = 1, 1, 0, "full"


def _run(monkeypatch, capsys):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setattr(bench, "CPU_SAMPLE", (3000, 1024, 30))
    assert bench.run_reference(_Args()) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "vectors/s" and line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": "vectors/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] == (os.cpu_count() or 1)
    assert "3000 x 1024 rows, 30 centres" in cb["sample"]
    # the same config object as the GPU arm's line, so the two lines compare
    assert line["config"] == bench.workload_config("full", 1)
    return line


def test_reference_arm_times_the_binary_where_it_runs(monkeypatch, capsys):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    line = _run(monkeypatch, capsys)
    want = "reference" if oracle.ref_binary(1024) and os.uname().machine == "x86_64" else None
    if want:
        assert line["cpu_baseline"]["kind"] == "reference"
        assert "unmodified reference binary" in line["note"]
    else:
        assert line["cpu_baseline"]["kind"] in ("reference", "port")


def test_reference_arm_falls_back_to_the_port(monkeypatch, capsys):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    monkeypatch.setattr(oracle, "ref_binary", lambda d=1024: None)
    line = _run(monkeypatch, capsys)
    assert line["cpu_baseline"]["kind"] == "port"
    assert "restatement" in line["note"]


def test_reference_arm_falls_back_when_the_binary_cannot_run(monkeypatch, capsys, tmp_path):
    """A binary of another architecture fails at exec (OSError): the arm takes the port."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    fake = tmp_path / "main"
    fake.write_bytes(b"\x7fELF not a runnable image")
    fake.chmod(0o755)
    monkeypatch.setattr(oracle, "ref_binary", lambda d=1024: str(fake))
    line = _run(monkeypatch, capsys)
    assert line["cpu_baseline"]["kind"] == "port"
