"""dnsmc_gb300 -- GB300-native reverse Monte Carlo radiative-source solver.

The hot path (per-cell OERM ray march) is CUDA for sm_103a in libdnsmc.so,
behind the C ABI of include/dnsmc.h; this package is its Python host mirror.
"""
from ._lib import (DnsmcError, LAYOUT_DENSE, LAYOUT_FORTRAN, MODEL_CK, MODEL_GREY, MODEL_GREY_BANDS,
                   MODEL_PARTICLE, MODEL_TABLE, RESULT_F32, RESULT_F64, SAMPLER_IID, SAMPLER_RQMC, STATUS_BAD_FIELD,
                   STATUS_COPY_TIMEOUT, STATUS_NONFINITE, STATUS_STEP_CAP)
from .api import (CvNet, Solver, ck_from_lbl, cvnet_default_config, default_config, dropin_configure, dropin_release,
                  get_results, mc_gpu, solver_rays_per_item)

__all__ = ["Solver", "CvNet", "ck_from_lbl", "cvnet_default_config", "solver_rays_per_item", "default_config", "mc_gpu", "get_results", "dropin_configure", "dropin_release",
           "DnsmcError", "MODEL_CK", "MODEL_GREY", "MODEL_GREY_BANDS", "MODEL_PARTICLE", "MODEL_TABLE",
           "LAYOUT_DENSE", "LAYOUT_FORTRAN", "SAMPLER_IID", "SAMPLER_RQMC", "STATUS_STEP_CAP", "STATUS_NONFINITE", "STATUS_BAD_FIELD",
           "STATUS_COPY_TIMEOUT", "RESULT_F64", "RESULT_F32"]
