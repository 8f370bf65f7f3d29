"""Pins the CPU oracle to the reference's own known-answer tests.

The reference ships no golden vectors; its pass/fail criteria are the
analytical checks in pydem/*.py and src/mesh.rs:146-172. The oracle passes
them at the reference's own precision (f32) and in FP64.
"""
import pytest

from tests import scenarios


@pytest.fixture(params=[32, 64], ids=["f32", "f64"])
def create(request, oracle_mod):
    prec = request.param

    def make(*args):
        return oracle_mod.OracleSimulation.create(*args, prec=prec)

    return make


@pytest.mark.parametrize("prec", [32, 64])
def test_triangle_intersection(oracle_mod, prec):
    scenarios.triangle_known_answer(lambda t, n, c, r: oracle_mod.triangle_query(t, n, c, r, prec))


def test_free_fall(create):
    scenarios.free_fall(create)


def test_hertzian_compression(create):
    scenarios.hertzian_compression(create)


def test_rolling_time(create, tmp_path):
    scenarios.rolling(create, str(tmp_path))


def test_jkr_pull_off(create):
    scenarios.jkr_pull_off(create)


def test_sjkr_pull_off(create):
    scenarios.sjkr_pull_off(create)


def test_contact_models(create):
    assert scenarios.contact_models(create, pytest.raises) == 0


def test_periodic(create):
    sim = scenarios.periodic_y(create)
    assert 0 < sim.get_particle_count() <= 101


def test_column_1000(create):
    sim = scenarios.column_1000(create)
    assert sim.get_particle_count() <= 1000
