"""The C ABI from plain C: ``tests/c_host/consumer.c`` includes only
``include/dmgs.h`` (compiled as strict C99, warnings as errors) and links
``libdmgs_gb300.so`` directly, as a non-Python host would.  It runs the
host-side paths (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

from dmgs_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_plain_c_host_links_and_runs(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    build()
    libdir = os.path.join(ROOT, "dmgs_gb300")
    exe = str(tmp_path / "consumer")
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_host", "consumer.c"),
                    "-L", libdir, "-ldmgs_gb300", "-Wl,-rpath," + libdir, "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "c consumer ok" in r.stdout
