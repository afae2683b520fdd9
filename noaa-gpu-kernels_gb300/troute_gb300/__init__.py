"""GB300-native Muskingum-Cunge secant routing (t-route MC path) over a C ABI."""
from .api import (  # noqa: F401
    CHPARAMS_DTYPE, CHPARAMS_F32_DTYPE, Cfg, Network, Stats, TrouteError, WarmModel, critical_path, device_info,
    exported_symbols, levels,
    read_network, write_network, linear_coeffs, linear_route, LinearNetwork, matrix_coeffs, matrix_route, MatrixNetwork, diffusive_tridiag, qlat_from_csv, write_forcings,
    debug_pow, debug_div, debug_quot_gt, measure_fp64_rate, lib, library_path, make_cfg, mc_reach_parallel, route_tree, timeout_probe, validate,
    wavefront_fp64)
from .hydrofabric import gpkg_to_network, read_gpkg  # noqa: F401
