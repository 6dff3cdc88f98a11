"""The product path has no CPU fallback (CPU): the binding, kernels and
driver never load, import or link the oracle (only build.py compiles it, as
test infrastructure), and the binding fails loudly when the CUDA library is
missing instead of answering some other way."""
from __future__ import annotations

import re
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpu-rmq_gb300"


def test_product_sources_do_not_use_the_oracle():
    offenders = []
    for p in sorted(list(PKG.glob("*.py")) + list((PKG / "csrc").glob("*")) + list((PKG / "driver").glob("*"))):
        if p.name == "build.py" or not p.is_file() or p.suffix in (".so", ".o"):
            continue
        text = p.read_text(errors="replace")
        if re.search(r"^\s*(from|import)\s+oracle\b|liboracle|oracle/|#include\s+\"[^\"]*oracle", text, re.M):
            offenders.append(p.name)
    assert not offenders, offenders


def test_binding_fails_loudly_without_the_library(tmp_path):
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import rmq_gb300 as R\n"
            "try:\n"
            "    R.lib()\n"
            "except RuntimeError as e:\n"
            "    print('raised', 'missing' in str(e))\n"
            "else:\n"
            "    print('loaded')\n") % str(PKG)
    env = {"RMQ_GB300_LIB": str(tmp_path / "absent" / "librmq_gb300.so"), "PATH": "/usr/bin:/bin"}
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)
    assert out.stdout.strip() == "raised True", out.stdout + out.stderr
