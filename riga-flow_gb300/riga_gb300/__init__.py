"""riga_gb300 — Python binding of the GB300 Monte Carlo engine's C ABI (include/riga_gb300.h).

The engine itself is native: CUDA kernels for sm_103a plus a C++ host layer behind an
``extern "C"`` boundary (``riga-flow_gb300/csrc``).  This package loads that in-tree library with
ctypes and mirrors the reference's public Rust API for the scenario hot path:

* ``price_put_leg`` — crates/riga-engine/src/lib.rs:183
* ``price_scenarios`` / ``price_risk_batch`` / ``price_central_greeks`` —
  crates/riga-risk/src/lib.rs:117-186, 573-626
* ``run_paths`` / ``reconstruct_path`` / ``query_worst_percentile`` —
  crates/riga-engine/src/explain.rs:90-372
* ``gpu`` — the ``gpu`` backend functions of crates/riga-engine/src/gpu.rs:500-564
"""
from .abi import RigaError  # noqa: F401
from .types import (EngineOptions, ImpliedVolGrid, MarketSnapshot, PhoenixTrade,  # noqa: F401
                    PriceRequest, SimulationConfig, VarianceReduction)

__all__ = ["RigaError", "EngineOptions", "ImpliedVolGrid", "MarketSnapshot", "PhoenixTrade",
           "PriceRequest", "SimulationConfig", "VarianceReduction"]
