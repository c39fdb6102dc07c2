"""GB300-native split-operator propagators with the interface of dibondar/AccurateWigner.

    from accuratewigner_gb300 import WignerMoyalCUDA1D, WignerBlochCUDA1D
    from accuratewigner_gb300 import RhoVNeumannCUDA1D, RhoBlochCUDA1D, SchrodingerWignerCUDA1D

The classes keep the reference's constructor keywords, attributes and methods;
the work runs in ``libawigner.so`` (C ABI in ``include/awigner.h``).
"""
from .wigner_moyal_cuda_1d import WignerMoyalCUDA1D
from .wigner_bloch_cuda_1d import WignerBlochCUDA1D
from .rho_vneumann_cuda_1d import RhoVNeumannCUDA1D
from .rho_bloch_cuda_1d import RhoBlochCUDA1D
from .schrodinger_wigner_cuda_1d import SchrodingerWignerCUDA1D
from ._common import check_config

__all__ = ["WignerMoyalCUDA1D", "WignerBlochCUDA1D", "RhoVNeumannCUDA1D", "RhoBlochCUDA1D", "SchrodingerWignerCUDA1D",
           "check_config"]
