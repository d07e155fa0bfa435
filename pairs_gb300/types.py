"""Type, shape, target and partitioner constants of the reference's public API
(src/pairs/__init__.py:24-67, sim/shapes.py, sim/flags.py, code_gen/target.py)."""


class Types:
    Invalid, Int32, Int64, UInt64, Float, Double, Boolean, String, Vector, Array, Matrix, Quaternion = range(12)
    Real = Double


class Shapes:
    Sphere = 0
    Halfspace = 1
    PointMass = 2


class Flags:
    Infinite = 1 << 0
    Ghost = 1 << 1
    Fixed = 1 << 2
    Global = 1 << 3


class DomainPartitioners:
    Regular = 0
    RegularXY = 1


class Target:
    Backend_CPP, Backend_CUDA = 0, 1
    Feature_CPU, Feature_GPU, Feature_OpenMP = 1, 5, 6

    def __init__(self, backend, features):
        self.backend = backend
        self.features = features if isinstance(features, list) else [features]

    def is_cpu(self):
        return self.Feature_CPU in self.features

    def is_gpu(self):
        return self.Feature_GPU in self.features

    def is_openmp(self):
        return self.Feature_OpenMP in self.features
