"""The reference's module name, bound to the GB300 implementation.

Scripts written against the reference (``import rusty_particles`` followed by
``rusty_particles.Simulation.create(...)``, src/lib.rs:24-35) run unchanged
against ``rusty_particles_gb300``: this package re-exports its public surface
(``Simulation``, ``set_num_threads``, ``hello``) under the reference's name.
Every step still runs on the GPU through librp.so; there is no CPU path.
"""
from rusty_particles_gb300 import (  # noqa: F401
    RP_MODE_PARITY,
    RP_MODE_PHYSICAL,
    RP_PREC_FP64,
    RP_PREC_MIXED,
    Simulation,
    hello,
    set_num_threads,
)

__all__ = ["Simulation", "set_num_threads", "hello", "RP_PREC_FP64", "RP_PREC_MIXED", "RP_MODE_PARITY",
           "RP_MODE_PHYSICAL"]
