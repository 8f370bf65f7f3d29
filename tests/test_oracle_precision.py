"""The oracle at the reference's precision (f32) against the oracle in FP64 on
the same bed for one step: forces agree to f32 rounding (median ~3e-6 of the
per-particle contact scale; the worst particle within 5e-4 for the linear and
Hertz laws, more for JKR and sJKR, whose Newton solve and cut-offs amplify
rounding), positions to one f32 rounding of the coordinates."""
import numpy as np
import pytest

from tests import parity_util as pu

LO, HI = (-0.25, -0.25, -0.25), (0.25, 0.25, 0.25)


def _step(oracle_mod, st, normal, prec, gamma):
    s = oracle_mod.OracleSimulation(1e-5, LO, HI, prec=prec)
    s.set_mode(0)
    s.set_cell_size(1.0)
    s.set_options(record_pairs=False, keep_contact_map=False)
    s.set_particle_material(1e7, 0.3, 2500.0, 0.5, 0.5, gamma)
    s._L.orc_set_models(s._h, normal, 0)
    s.set_periodic_boundary(False, False, False)
    for i in range(len(st["radius"])):
        p = st["position"][i]
        s.add_particle(p[0], p[1], p[2], st["radius"][i], st["mass"][i], bool(st["fixed"][i]))
    s.set_state({"x": st["position"], "v": st["velocity"], "a": st["acceleration"], "w": st["angular_velocity"],
                 "tau": st["torque"]})
    s.step()
    F, _ = s.last_forces()
    FS, _ = s.last_force_scale()
    return F, FS, s.state()["x"]


@pytest.mark.parametrize("normal,worst", [(0, 5e-4), (1, 5e-4), (3, 2e-2), (4, 5e-3)])
def test_f32_oracle_tracks_fp64(oracle_mod, normal, worst):
    st = pu.random_bed(300 + normal, 2000, LO, HI, 0.008, 0.012)
    gamma = 0.05 if normal in (3, 4) else 0.0
    F32, _, x32 = _step(oracle_mod, st, normal, 32, gamma)
    F64, FS, x64 = _step(oracle_mod, st, normal, 64, gamma)
    touched = FS > 0
    err = np.linalg.norm(F32 - F64, axis=1)[touched] / FS[touched]
    assert np.median(err) < 1e-5
    assert err.max() < worst
    assert np.all(np.abs(x32 - x64) <= 2.0 ** -23 * np.abs(x64) + 1e-12)
