"""GB300-native scalar-propagation hot path of FluxOptics.jl.

Import name: ``fluxoptics_gb300`` (loaded from this directory by
``__graft_entry__.load_package``).  Device arrays are CUDA tensors; every
operation runs through libfluxoptics_gb300 (hand-written sm_103a kernels) and
fails loudly when the library cannot be loaded.
"""

from . import _capi
from ._capi import FluxOpticsError
from .build import build as build_library
from .components import (AS_BPM, ASProp, ASPropZ, Backward, Component, FieldProbe, FourierMask, FourierOperator, FourierPhase,
                         FourierWrapper, Forward, Mask, OpticalSequence, OpticalSystem, PadCropOperator, ParaxialProp, Phase,
                         RSProp, TiltAnchor, adjoint, crop, pad,
                         ScalarSource, TeaDOE, TeaReflector, backpropagate, backpropagate_, function_to_array,
                         get_components, get_data, get_sequence, get_source, isbuffered, istrainable, propagate, propagate_,
                         reverse, spatial_vectors, trainable)
from .fields import (ScalarField, coupling_efficiency, dot, get_lambdas, get_lambdas_collection, get_tilts,
                     get_tilts_collection, intensity, is_on_axis, normalize_power_, offset_tilts_, phase, power,
                     select_lambdas, select_tilts, set_field_data, set_field_ds_, set_field_tilts)
from .metrics import (DotProduct, PowerCoupling, SquaredFieldDifference, SquaredIntensityDifference,
                      backpropagate_metric, compute_metric, withgradient)
from .modes import (Gaussian, Gaussian1D, HermiteGaussian, HermiteGaussian1D, LaguerreGaussian, gaussian,
                    hermite_gaussian,
                    hermite_gaussian_groups)
from .optimisers import (ClampProx, Descent, Fista, IstaProx, Momentum, Nesterov, NoDescent, PointwiseProx,
                         PositiveProx, ProxRule,
                         TVProx, make_rules, setup, tv_denoise_, update_)
from .ragged import RaggedBatch

load_library = _capi.load

__all__ = [
    "ASProp", "ASPropZ", "AS_BPM", "Backward", "ClampProx", "Component", "Descent", "DotProduct", "FieldProbe", "Fista", "FluxOpticsError", "FourierMask", "FourierOperator", "FourierPhase", "FourierWrapper",
    "Forward", "Gaussian", "Gaussian1D", "HermiteGaussian", "HermiteGaussian1D", "LaguerreGaussian", "IstaProx", "Mask", "Momentum", "Nesterov", "NoDescent", "OpticalSequence", "OpticalSystem", "PadCropOperator", "ParaxialProp", "Phase", "PointwiseProx", "PositiveProx", "PowerCoupling", "ProxRule",
    "RSProp", "RaggedBatch", "ScalarField", "ScalarSource", "SquaredFieldDifference", "SquaredIntensityDifference", "TVProx", "TeaDOE",
    "TeaReflector", "TiltAnchor", "adjoint", "backpropagate", "backpropagate_metric", "compute_metric", "crop", "pad", "backpropagate_", "get_components", "get_data", "get_sequence", "get_source", "isbuffered",
    "istrainable", "trainable", "build_library", "coupling_efficiency", "dot", "function_to_array", "get_lambdas", "get_lambdas_collection", "get_tilts",
    "get_tilts_collection", "is_on_axis", "offset_tilts_", "phase", "select_lambdas", "select_tilts", "set_field_data", "set_field_ds_",
    "set_field_tilts", "gaussian",
    "hermite_gaussian", "hermite_gaussian_groups", "intensity", "load_library", "make_rules",
    "normalize_power_", "power", "propagate", "propagate_", "reverse", "setup", "spatial_vectors", "tv_denoise_", "update_",
    "withgradient",
]
