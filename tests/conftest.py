"""Test configuration: registers the `gpu` marker and makes the package importable.

The package directory is `dynamiclighting-bevy_gb300/` (not a Python identifier), so it is
loaded under the name `dynlight_gb300`.
"""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    if "dynlight_gb300" in sys.modules:
        return sys.modules["dynlight_gb300"]
    pkg_dir = os.path.join(ROOT, "dynamiclighting-bevy_gb300")
    spec = importlib.util.spec_from_file_location(
        "dynlight_gb300", os.path.join(pkg_dir, "__init__.py"),
        submodule_search_locations=[pkg_dir])
    module = importlib.util.module_from_spec(spec)
    sys.modules["dynlight_gb300"] = module
    spec.loader.exec_module(module)
    return module


load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
