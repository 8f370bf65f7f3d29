"""The reference's module name and call surface, checked without a GPU.

``import rusty_particles`` must resolve to this product, and every call the
reference's own Python scripts make (pydem/*.py: Simulation.create, the
Simulation methods, the module functions) must exist on it with an argument
list that accepts the call. The scripts themselves step simulations, which
needs a GPU; they are read here as text (when the reference checkout is on
this machine) to collect the calls.
"""
import ast
import inspect
import os

import pytest

import rusty_particles
import rusty_particles_gb300

REF_PYDEM = "/root/reference/pydem"


def test_module_name_resolves_to_the_product():
    assert rusty_particles.Simulation is rusty_particles_gb300.Simulation
    assert rusty_particles.set_num_threads is rusty_particles_gb300.set_num_threads
    assert isinstance(rusty_particles.hello(), str)


def _calls(tree):
    """(receiver, method, positional count, keyword names) of every attribute call."""
    out = []
    for node in ast.walk(tree):
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute):
            recv = node.func.value
            name = recv.id if isinstance(recv, ast.Name) else (
                f"{recv.value.id}.{recv.attr}" if isinstance(recv, ast.Attribute) and isinstance(recv.value, ast.Name)
                else None)
            out.append((name, node.func.attr, len(node.args), [k.arg for k in node.keywords if k.arg]))
    return out


@pytest.mark.skipif(not os.path.isdir(REF_PYDEM), reason="reference scripts not on this machine")
def test_reference_scripts_calls_exist():
    seen = 0
    for fn in sorted(os.listdir(REF_PYDEM)):
        if not fn.endswith(".py"):
            continue
        tree = ast.parse(open(os.path.join(REF_PYDEM, fn)).read())
        # names bound to a Simulation (x = rusty_particles.Simulation.create(...))
        sims = set()
        for node in ast.walk(tree):
            if isinstance(node, ast.Assign) and isinstance(node.value, ast.Call):
                f = node.value.func
                if isinstance(f, ast.Attribute) and f.attr == "create":
                    sims.update(t.id for t in node.targets if isinstance(t, ast.Name))
        for recv, meth, npos, kws in _calls(tree):
            if recv == "rusty_particles":
                target = getattr(rusty_particles, meth)
            elif recv == "rusty_particles.Simulation":
                target = getattr(rusty_particles.Simulation, meth)
            elif recv in sims:
                target = getattr(rusty_particles.Simulation, meth)
                npos += 1  # self
            else:
                continue
            sig = inspect.signature(target)
            sig.bind(*([None] * npos), **{k: None for k in kws})
            seen += 1
    assert seen >= 40
