"""dachshund-gb300: Dachshund's Wiener-filter hot path on one GB300 (sm_103a).

Signal covariance (table or exact), the SN / W operators, Jacobi-PCG and the
map projection, as hand-written CUDA kernels behind the C ABI of
``include/ds_gb300.h``.  See ``api`` for the Python face of that ABI.
"""
from .api import (  # noqa: F401
    BatchResult,
    BatchSolver,
    Context,
    MapGrid,
    MixedParams,
    PCGParams,
    PCGResult,
    SignalCovarParams,
    WFVectorSN,
    WFVectorW,
    init_uniform_map_coords,
    map_covar_diag,
    npixel_to_pixel,
    pixel_to_npixel,
    pixel_to_wpixel,
    points_from_pixels,
    read_pixel_data,
    sigma_m_noise_dom,
    signal_covar,
    smp_product,
    solve_cf,
    table_init,
    wpixel_to_pixel,
)
from ._lib import DsError  # noqa: F401
from .build import build  # noqa: F401
