"""Test helpers that load the product binding (cmm-turbulence_gb300/cmm.py)."""
import importlib.util
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cmm-turbulence_gb300")


def cmm():
    if "cmm_gb300" in sys.modules:
        return sys.modules["cmm_gb300"]
    build = _load("cmm_gb300_build", os.path.join(PKG, "build.py"))
    build.build()
    return _load("cmm_gb300", os.path.join(PKG, "cmm.py"))


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def header_functions():
    """Names of every function declared in include/cmm_abi.h."""
    import re
    text = open(os.path.join(ROOT, "include", "cmm_abi.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cmm_[a-z_0-9]+)\s*\(", text)))


def read_monitoring(run_dir):
    """Load every .data file under Monitoring_data like the reference harness
    (tests/test_functions.py:98-118) -> {relative name: list of float}."""
    import numpy as np
    out = {}
    base = os.path.join(run_dir, "Monitoring_data")
    for root, _, files in os.walk(base):
        for fn in files:
            if fn.endswith(".data") and not fn.endswith("_Hash.data") and fn != "Time_c.data":
                rel = os.path.relpath(os.path.join(root, fn), base)[: -len(".data")]
                out[rel] = list(np.fromfile(os.path.join(root, fn), dtype="<f8"))
    return out
