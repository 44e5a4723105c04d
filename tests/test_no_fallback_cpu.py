"""The product path has no CPU fallback: without the CUDA library it fails
loudly, and nothing in the package reaches for the oracle."""
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "edxraster_gb300")


def test_renderer_without_the_library_raises(tmp_path):
    # a copy of the package sources with no built library beside them
    shutil.copytree(PKG, tmp_path / "edxraster_gb300", ignore=shutil.ignore_patterns("_build", "__pycache__"))
    code = ("import edxraster_gb300.renderer as R\n"
            "try:\n"
            "    R.Renderer()\n"
            "except ImportError as e:\n"
            "    print('raised:', e)\n"
            "else:\n"
            "    raise SystemExit('rendered without libedxr.so')\n")
    env = dict(os.environ, PYTHONPATH=str(tmp_path))
    out = subprocess.run([sys.executable, "-c", code], cwd=tmp_path, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "raised:" in out.stdout and "not built" in out.stdout


def test_package_never_imports_the_oracle():
    for dirpath, _, files in os.walk(PKG):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, fn), errors="replace").read()
                assert "import oracle" not in text and "from oracle" not in text, fn
                assert "edxr_oracle" not in text and "pyoracle" not in text, fn
