"""GB300-native (sm_103a) hot path of the SSshuishui/viss_recon_shade simulator.

Lunar-orbit satellite positions and baseline uvw, Moon shade windows, the
shaded direct visibility DFT and the direct-DFT reconstruction, as
hand-written CUDA kernels behind the C ABI of libvissgb.so
(include/viss_gb300.h); this package is the Python host side over that ABI.
"""
from .api import (ChannelBatch, DftConfig, OrbitConfig, Tuning, autotune, autotune_report,  # noqa: F401
                  baseline_uvw, dedup_uvw, imagerecon, normalise_shade, nxq, orbit_positions, recon, recon_ratios,
                  reference_d, shade_windows, tuning_candidates, unique_uvw, vis_dft, vis_dft_map, vis_dft_windowed,
                  visscal)
from ._lib import (MASK_GEOMETRIC, MASK_NONE, MASK_REF_INTENDED, MASK_REF_QUIRK, PREC_COMPENSATED,  # noqa: F401
                   PREC_F64_PHASE, PREC_FAST, PREC_PLAIN, RECON_MASK_GEOMETRIC, RECON_MASK_NONE, RECON_MASK_REF, VARIANT_OPTIM,
                   VARIANT_PLAIN, VissError)
