"""The committed algorithmic-bytes fixture (tests/golden/algorithmic_bytes.json)
re-derived from the oracle, so the roofline's bytes per ray cannot go stale
when a workload generator or the oracle's traversal counts change."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def committed():
    return json.load(open(os.path.join(HERE, "golden", "algorithmic_bytes.json")))


def _fixtures():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_fixtures", os.path.join(HERE, "golden", "make_fixtures.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_closest_bytes_fixture(committed):
    assert _fixtures().closest_bytes() == committed["closest"]


def test_path_tracing_bytes_fixtures(committed):
    m = _fixtures()
    assert m.box_scene_bytes() == committed["pt_box"]
    assert m.knot_bytes() == committed["pt_knot"]
