"""Where the reference checkout lies, for the scripts that build or run it
(test infrastructure only).  The environment variable SCLET_REFERENCE_ROOT
wins; otherwise the default of the build recipe oracle/Makefile.ref, the one
place that names the build host's mount point."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_root() -> str:
    env = os.environ.get("SCLET_REFERENCE_ROOT")
    if env:
        return env
    try:
        r = subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref", "print-ref-root"], cwd=ROOT,
                           capture_output=True, text=True, timeout=60)
        return r.stdout.strip() if r.returncode == 0 else ""
    except Exception:
        return ""


def omega_sources() -> str:
    """The beta->omega driver's sources, or "" when no checkout is present."""
    root = reference_root()
    d = os.path.join(root, "source_beta_to_omega") if root else ""
    return d if d and os.path.isdir(d) else ""
