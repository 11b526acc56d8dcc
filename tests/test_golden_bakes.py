"""The committed golden bakes (tests/golden/bakes.json, written from the oracle by
tests/golden/make_golden.py): the oracle reproduces them on this machine's CPU, at any thread
count, and every CUDA form reproduces them on the GPU. The fixtures were made on one machine and
are checked on others, so they also pin the oracle and the CUDA bake across hosts (x86-64 and
aarch64). Digests are of integer words and float bit patterns: the bar is bit-exact."""
import json
import os

import pytest

import dynlight_gb300 as dl

from .golden import cases

with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bakes.json")) as _f:
    GOLDEN = json.load(_f)["cases"]


def _expected(name):
    want = dict(GOLDEN[name])
    want.pop("oracle_seconds", None)
    return want


def test_every_case_has_a_fixture():
    assert sorted(GOLDEN) == sorted(cases.CASES)


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_oracle_reproduces_the_golden_bake(name):
    assert cases.digest(cases.oracle_bake(name)) == _expected(name)


@pytest.mark.parametrize("name", ["mixed_lights", "root_leaf", "colored_mixed_bounce"])
def test_oracle_golden_bake_on_one_thread(name):
    # the oracle's reductions are commutative: one thread gives the many-thread bytes
    assert cases.digest(cases.oracle_bake(name, threads=1)) == _expected(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_cuda_forms_reproduce_the_golden_bake(name):
    inp, opts, form = cases.CASES[name]()
    want = _expected(name)
    forms = ["refined"] if form == "refined" else ["batched", "plain"]
    for f in forms:
        assert cases.digest(dl.bake(inp, opts, form=f)) == want, f
