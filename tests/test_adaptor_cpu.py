"""The reference-side adaptors (opensph_gb300/adaptor) compile against the reference's own headers and link
with its core library and libsphgpu.so; without a GPU the drop-in reports the missing device through the
reference's exception type. Runs only where the reference tree and its built core library exist."""
import os
import subprocess

import pytest

from opensph_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference tree: oracle/Makefile's REF (OPENSPH_REFERENCE when set)
REF = subprocess.run(["make", "-s", "--no-print-directory", "-C", os.path.join(REPO, "oracle"), "print-ref"],
                     capture_output=True, text=True).stdout.strip()
LIBCORE = os.path.join(REPO, "oracle", "_ref", "libcore.a")


@pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "core")) and os.path.exists(LIBCORE)),
                    reason="reference tree or its built core library not present")
def test_adaptor_builds_and_reports_missing_device(tmp_path):
    if not os.path.exists(abi.LIBRARY_PATH):
        pytest.skip("libsphgpu.so is not built")
    exe = tmp_path / "adaptor_check"
    src = os.path.join(REPO, "opensph_gb300", "adaptor")
    cmd = ["g++", "-std=c++14", "-O1", "-msse4.1", "-pthread", "-w", "-I", os.path.join(REF, "core"),
           "-I", os.path.join(REPO, "include"), os.path.join(src, "GpuSph.cpp"), os.path.join(src, "adaptor_check.cpp"),
           LIBCORE, abi.LIBRARY_PATH, "-Wl,-rpath," + os.path.dirname(abi.LIBRARY_PATH), "-o", str(exe)]
    subprocess.run(cmd, check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode in (0, 3), res.stdout + res.stderr
    if res.returncode == 3:
        assert "no CUDA device" in res.stdout


@pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "core")) and os.path.exists(LIBCORE)),
                    reason="reference tree or its built core library not present")
def test_adaptor_syncs_device_state_only_for_output(tmp_path):
    # GpuTimeStepping (ON_DEMAND) + GpuOutput around the reference's BinaryOutput, with a host-memory stand-in
    # for libsphgpu (tests/adaptor/fake_sphgpu.cpp) that counts transfers; the dump is read back with the
    # reference's BinaryInput
    exe = tmp_path / "adaptor_sync_check"
    src = os.path.join(REPO, "opensph_gb300", "adaptor")
    here = os.path.join(REPO, "tests", "adaptor")
    cmd = ["g++", "-std=c++14", "-O1", "-msse4.1", "-pthread", "-w", "-I", os.path.join(REF, "core"),
           "-I", os.path.join(REPO, "include"), "-I", src, os.path.join(src, "GpuSph.cpp"),
           os.path.join(here, "adaptor_sync_check.cpp"), os.path.join(here, "fake_sphgpu.cpp"), LIBCORE,
           "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = tmp_path / "out"
    out.mkdir()
    res = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "ok" in res.stdout
    assert any(p.suffix == ".ssf" for p in out.iterdir())
