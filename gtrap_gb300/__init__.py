"""gtrap_gb300 -- GB300-native (sm_103a) batched transit search.

Drop-in modules mirroring the reference package ``gtrap``:

* :mod:`gtrap_gb300.geebls`        -- masked BLS (``gbls_module``)
* :mod:`gtrap_gb300.geebls_simple` -- plain BLS (``gbls_module``)
* :mod:`gtrap_gb300.gtls`          -- trapezoid least squares (``gtls_module``)
* :mod:`gtrap_gb300.gfilter`       -- median detrend (``gmf_module``, ``get_detrend``, ``get_offset``)
* :mod:`gtrap_gb300.getstat`       -- BLS peak statistics (``get_blsstat``)
* :mod:`gtrap_gb300.tls`           -- trapezoid grid fit (``gen_trapzoid``, ``get_chi2Hmax``, ``tlsfit``)
* :mod:`gtrap_gb300.detect_peaks`  -- ``detect_peaks``
* :mod:`gtrap_gb300.picktrap`      -- ``pick_Wnormalized_cleaned_lc_direct``
* :mod:`gtrap_gb300.genmock`       -- ``gentransit``, ``gensin``, ``gendcos``
* :mod:`gtrap_gb300.ggenmock`      -- ``gabcrm_module`` (the gamma sampler)
* :mod:`gtrap_gb300.driver`        -- ``pycuda.driver``-style allocation and copies

:mod:`gtrap_gb300.api` is the tensor-level interface; all computation runs in the
native library ``gtrap_gb300/_lib/libgtrap_gb300.so`` (C ABI: ``include/gtrap_gb300.h``).
"""
from . import _native
from ._native import GtrapError

__all__ = ["GtrapError", "api", "driver", "geebls", "geebls_simple", "gtls", "gfilter", "getstat",
           "batch", "serve", "tls", "detect_peaks", "picktrap", "genmock", "ggenmock"]

__version__ = "0.1.0"


def __getattr__(name):
    # Submodules import torch; load them on first access so that importing the package
    # (e.g. to inspect the native library) stays cheap.
    if name in {"api", "driver", "geebls", "geebls_simple", "gtls", "gfilter", "getstat", "batch",
                "serve", "tls", "detect_peaks", "picktrap", "genmock", "ggenmock"}:
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
