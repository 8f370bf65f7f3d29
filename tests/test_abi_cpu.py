"""Host-side checks of librp.so that need no GPU: the library builds, loads and
exports every entry point include/rp.h declares; the binding maps error codes
to the reference's exception types; host-only calls (model names, STL
loading, getters before the first step, VTK output) behave like the
reference's; stepping without a GPU fails loudly instead of falling back.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import rusty_particles_gb300 as rp
from rusty_particles_gb300 import _lib
from tests.stl_util import floor_tris, write_ascii_stl, write_binary_stl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "rp.h")).read()
    return sorted(set(re.findall(r"\b(rp_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    syms = header_symbols()
    assert len(syms) >= 30
    assert set(syms) == set(_lib.SIGNATURES), set(syms) ^ set(_lib.SIGNATURES)


def test_library_exports_every_symbol():
    L = _lib.load()
    for s in header_symbols():
        assert hasattr(L, s), s


def test_version_string():
    assert b"sm_103a" in _lib.load().rp_version()


def test_contact_model_names():
    sim = rp.Simulation.create(0.001, -1.0, 0.0, -1.0, 1.0, 5.0, 1.0, 100)
    for n in ["hertz", "Hertzian", "LINEAR", "spring_dashpot", "hysteretic", "jkr", "sJKR", "simplified_jkr"]:
        for t in ["mindlin", "Coulomb", "linear", "spring_coulomb"]:
            sim.set_contact_models(n, t)
    with pytest.raises(ValueError):
        sim.set_contact_models("invalid", "coulomb")
    with pytest.raises(ValueError):
        sim.set_contact_models("hertz", "invalid")


def test_getters_setters_and_index_errors():
    sim = rp.Simulation.create(0.001, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 10)
    sim.add_particle(0.1, 0.2, 0.3, 0.05, 1.0)
    sim.add_particle(-0.1, 0.0, 0.0, 0.05, 1.0, fixed=True)
    assert sim.get_particle_count() == 2
    assert sim.get_particle_position(0) == (0.1, 0.2, 0.3)
    sim.set_particle_velocity(1, 1.0, 2.0, 3.0)
    assert sim.get_particle_velocity(1) == (1.0, 2.0, 3.0)
    sim.set_particle_angular_velocity(0, 0.0, 0.0, 5.0)
    assert sim.get_particle_angular_velocity(0) == (0.0, 0.0, 5.0)
    for fn in (sim.get_particle_position, sim.get_particle_velocity, sim.get_particle_angular_velocity):
        with pytest.raises(IndexError):
            fn(2)
    with pytest.raises(IndexError):
        sim.set_particle_velocity(5, 0, 0, 0)
    st = sim.get_state()
    assert st["fixed"].tolist() == [0, 1]
    assert np.allclose(st["radius"], 0.05)


def test_stl_binary_ascii_and_errors(tmp_path):
    sim = rp.Simulation.create(0.001, -10.0, 0.0, -10.0, 10.0, 10.0, 10.0, 1)
    b = tmp_path / "floor.stl"
    write_binary_stl(str(b), floor_tris())
    sim.add_mesh(str(b))
    a = tmp_path / "floor_ascii.stl"
    write_ascii_stl(str(a), floor_tris())
    sim.add_mesh(str(a))
    with pytest.raises(IOError):
        sim.add_mesh(str(tmp_path / "missing.stl"))
    bad = tmp_path / "bad.stl"
    bad.write_bytes(b"\x00" * 80 + (5).to_bytes(4, "little") + b"\x00" * 10)
    with pytest.raises(IOError):
        sim.add_mesh(str(bad))


def test_vtk_format(tmp_path):
    sim = rp.Simulation.create(0.001, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 2)
    sim.add_particle(0.1, 0.25, -0.5, 0.05, 1.0)
    sim.add_particle(1e-7, 2.0, 3.0, 0.125, 1.0)
    path = tmp_path / "out.vtk"
    sim.write_vtk(str(path))
    lines = path.read_text().splitlines()
    assert lines[:5] == ["# vtk DataFile Version 3.0", "DEM Simulation Data", "ASCII", "DATASET POLYDATA",
                         "POINTS 2 float"]
    assert lines[5] == "0.1 0.25 -0.5"
    assert lines[6] == "0.0000001 2 3"
    assert lines[7:10] == ["POINT_DATA 2", "VECTORS velocity float", "0 0 0"]
    assert lines[11:15] == ["SCALARS radius float 1", "LOOKUP_TABLE default", "0.05", "0.125"]
    assert lines[15:19] == ["SCALARS id int 1", "LOOKUP_TABLE default", "0", "1"]
    with pytest.raises(IOError):
        sim.write_vtk(str(tmp_path / "no_such_dir" / "x.vtk"))


def test_invalid_arguments():
    with pytest.raises(ValueError):
        rp.Simulation.create(0.0, -1, -1, -1, 1, 1, 1, 1)
    sim = rp.Simulation.create(0.001, -1, -1, -1, 1, 1, 1, 1)
    with pytest.raises(ValueError):
        sim.set_particle_material(1e7, 0.3, 2500.0, -0.5, 0.5)
    with pytest.raises(ValueError):
        sim.set_precision(7)
    with pytest.raises(ValueError):
        sim.set_interaction_mode(9)


def test_hello_and_mpi_noop():
    assert isinstance(rp.hello(), str)
    sim = rp.Simulation.create(0.001, -1, -1, -1, 1, 1, 1, 1)
    assert sim.init_mpi() is None


def test_no_gpu_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sim = rp.Simulation.create(0.001, -1, -1, -1, 1, 1, 1, 1)
    sim.add_particle(0.0, 0.0, 0.0, 0.1, 1.0)
    with pytest.raises(RuntimeError):
        sim.enable_gpu()
    with pytest.raises(RuntimeError):
        sim.step()
    with pytest.raises(RuntimeError):
        sim.run(0.01)


def test_get_state_into_caller_arrays():
    sim = rp.Simulation.create(0.001, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 10)
    sim.add_particle(0.1, 0.2, 0.3, 0.05, 1.0)
    sim.add_particle(-0.1, 0.0, 0.0, 0.07, 2.0, fixed=True)
    fresh = sim.get_state()
    out = {k: np.full_like(v, 7) for k, v in fresh.items()}
    got = sim.get_state(out=out)
    assert got is out
    for k in fresh:
        np.testing.assert_array_equal(out[k], fresh[k])
    part = {"position": np.zeros((2, 3))}
    sim.get_state(out=part)
    np.testing.assert_array_equal(part["position"], fresh["position"])
    with pytest.raises(ValueError):
        sim.get_state(out={"position": np.zeros((3, 3))})
    with pytest.raises(ValueError):
        sim.get_state(out={"radius": np.zeros(2, np.float32)})
    with pytest.raises(ValueError):
        sim.get_state(out={"position": np.zeros((3, 2)).T})
    with pytest.raises(KeyError):
        sim.get_state(out={"speed": np.zeros((2, 3))})


def test_set_state_checks_lengths():
    sim = rp.Simulation.create(0.001, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 10)
    sim.add_particle(0.1, 0.2, 0.3, 0.05, 1.0)
    sim.add_particle(-0.1, 0.0, 0.0, 0.07, 2.0)
    sim.set_state({"velocity": np.ones((2, 3)), "mass": np.array([1.5, 2.5])})
    assert sim.get_particle_velocity(1) == (1.0, 1.0, 1.0)
    assert sim.get_state()["mass"].tolist() == [1.5, 2.5]
    for bad in ({"velocity": np.ones((1, 3))}, {"position": np.ones(6)}, {"radius": np.ones(3)},
                {"fixed": np.ones((2, 3), np.uint8)}):
        with pytest.raises(ValueError):
            sim.set_state(bad)
    with pytest.raises(KeyError):
        sim.set_state({"speed": np.ones((2, 3))})
    # the C ABI itself rejects a length other than the particle count
    L = _lib.load()
    st = _lib.RpState()
    v = np.ones((3, 3))
    st.n_particles = 3
    st.velocity = v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert L.rp_write_state(sim._h, ctypes.byref(st)) == _lib.RP_E_INVALID_ARG
    assert L.rp_read_state(sim._h, ctypes.byref(st)) == _lib.RP_E_INVALID_ARG
    assert sim.get_particle_velocity(1) == (1.0, 1.0, 1.0)
