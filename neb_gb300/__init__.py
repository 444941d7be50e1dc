"""neb_gb300: GB300-native (sm_103a) neural-eigenfluid hot path.

Jet MLP basis with analytic spatial derivatives, weighted mass / stiffness
Grams, FP64 generalized eigensolve with the spectral objective, and the
hand-written reverse pass -- CUDA kernels behind a C ABI
(include/neb_gb300.h), driven from PyTorch host code.
"""
from .configs import CONFIGS, NebConfig, sample, objective_weights
from .jets import Jet, pack, unpack
from .model import Model, SpectralObjective, SpectralResult, spectral_step, train_step
from .modes import ModeModel, coefficient_peel, velocity_step
from .hardcoded import HardcodedModel
from . import hardcoded
from .training import cosine_learning_rate, train, velocity_train_step

__all__ = ["CONFIGS", "NebConfig", "sample", "objective_weights", "Jet", "pack", "unpack",
           "Model", "SpectralObjective", "SpectralResult", "spectral_step", "train_step",
           "ModeModel", "coefficient_peel", "velocity_step", "cosine_learning_rate", "train",
           "velocity_train_step", "HardcodedModel", "hardcoded"]
