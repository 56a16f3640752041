"""Host-side checks of the reference-style driver that need no GPU: missing
and malformed run files are reported before any device work."""
import os
import subprocess

from rtm_gpu_gb300 import _build, capi


def test_missing_run_file(product_lib, tmp_path):
    rc = capi.lib().rtm_run_config(str(tmp_path / "none.txt").encode(), 0)
    assert rc == -6  # RTM_ERR_IO
    assert b"cannot open" in capi.lib().rtm_last_error()


def test_truncated_run_file(product_lib, tmp_path):
    p = tmp_path / "2D_Real_RVSP_RTM.txt"
    p.write_text("The maximum length of operator\n8\nThe minimum length\n2\n")
    assert capi.lib().rtm_run_config(str(p).encode(), 0) == -1  # RTM_ERR_ARG
    assert b"missing entries" in capi.lib().rtm_last_error()


def test_executable_reports_errors(product_lib, tmp_path):
    r = subprocess.run([_build.CLI], cwd=str(tmp_path), capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "2D_Real_RVSP_RTM.txt" in r.stderr


def test_window_outside_image_rejected(product_lib, tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import cli_case
    c = cli_case.default_case(NX_ED=61)  # beyond the 60-column image
    cli_case.write_case(str(tmp_path), c)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        rc = capi.lib().rtm_run_config(b"2D_Real_RVSP_RTM.txt", 0)
    finally:
        os.chdir(cwd)
    assert rc == -1 and b"output window" in capi.lib().rtm_last_error()
