"""pairs_gb300: the P4IRS particle hot path on one GB300 GPU.

Public API mirrors the reference package `pairs` (src/pairs/__init__.py:9-67):
simulation(), target_cpu()/target_gpu(), type and shape constants.  The compute path
is hand-written CUDA (libpairs_gb300.so) reached through a C ABI; there is no CPU
fallback.
"""
from .types import DomainPartitioners, Flags, Shapes, Target, Types

__all__ = ["simulation", "target_cpu", "target_gpu", "int32", "float", "double", "real", "vector",
           "matrix", "quaternion", "point_mass", "sphere", "halfspace", "regular_domain_partitioner",
           "regular_domain_partitioner_xy"]


def simulation(ref, shapes, dims=3, timesteps=100, double_prec=False, use_contact_history=False,
               particle_capacity=800000, neighbor_capacity=100, debug=False, **gb300_options):
    """Same signature as the reference's pairs.simulation(); extra keyword options:
    precision ("fp64" | "mixed"), ghost_sync ("reference" | "exact"),
    rebuild_policy ("fixed" | "guard" | "fixed+guard" | "learned"), device."""
    from .sim import Simulation
    return Simulation(ref, shapes, dims, timesteps, double_prec, use_contact_history, particle_capacity,
                      neighbor_capacity, debug, **gb300_options)


def target_cpu(parallel=False):
    if parallel:
        return Target(Target.Backend_CPP, [Target.Feature_CPU, Target.Feature_OpenMP])
    return Target(Target.Backend_CPP, Target.Feature_CPU)


def target_gpu():
    return Target(Target.Backend_CUDA, Target.Feature_GPU)


def int32():
    return Types.Int32


def float():  # noqa: A001 - the reference exports this name
    return Types.Float


def double():
    return Types.Double


def real():
    return Types.Real


def vector():
    return Types.Vector


def matrix():
    return Types.Matrix


def quaternion():
    return Types.Quaternion


def point_mass():
    return Shapes.PointMass


def sphere():
    return Shapes.Sphere


def halfspace():
    return Shapes.Halfspace


def regular_domain_partitioner():
    return DomainPartitioners.Regular


def regular_domain_partitioner_xy():
    return DomainPartitioners.RegularXY
