"""The drop-in command line's host-side paths, which need no GPU: the
default directory (inv.cu:26-29), a missing model failing loudly, and a
mode the reference's switch has no case for (inv.cu:33-90: nothing runs,
exit 0, only the config load's output directory is made)."""
import subprocess


def run(pkg, args, cwd):
    return subprocess.run([pkg.GBINV_PATH] + list(args), capture_output=True, text=True, timeout=60, cwd=cwd)


def test_default_directory_and_missing_model(pkg, tmp_path):
    r = run(pkg, [], str(tmp_path))
    assert r.stdout.startswith("Using default directory example/checker")
    assert r.returncode != 0
    assert "model_true/proc000000_x.bin" in r.stderr


def test_missing_model_fails_loudly(pkg, tmp_path):
    r = run(pkg, [str(tmp_path), "-mode=0"], str(tmp_path))
    assert r.returncode != 0
    assert "cannot open" in r.stderr and str(tmp_path) in r.stderr


def test_mode_without_a_case_does_nothing(pkg, tmp_path):
    (tmp_path / "config.ini").write_text("[global]\nmode = 9\n")
    r = run(pkg, [str(tmp_path)], str(tmp_path))
    assert r.returncode == 0
    assert r.stdout == "" and r.stderr == ""
    # the config load itself creates output/, empty (lib/config.h:101-104)
    assert (tmp_path / "output").is_dir() and not any((tmp_path / "output").iterdir())


def test_clean_flag_empties_output(pkg, tmp_path):
    """clean = 1 removes output/ before it is made again; clean = 0 keeps
    what is there (lib/config.h:101-104)."""
    (tmp_path / "output").mkdir()
    (tmp_path / "output" / "keep.bin").write_bytes(b"x")
    (tmp_path / "config.ini").write_text("[global]\nmode = 9\nclean = 0\n")
    assert run(pkg, [str(tmp_path)], str(tmp_path)).returncode == 0
    assert (tmp_path / "output" / "keep.bin").exists()
    (tmp_path / "config.ini").write_text("[global]\nmode = 9\nclean = 1\n")
    assert run(pkg, [str(tmp_path)], str(tmp_path)).returncode == 0
    assert (tmp_path / "output").is_dir() and not any((tmp_path / "output").iterdir())
