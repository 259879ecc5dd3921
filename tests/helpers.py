"""Shared helpers for the GPU tests."""

import os


def engine_with_variant(inp, variant):
    """Create an Engine with the kernel family forced by FWGB_VARIANT ("march" or "direct")."""
    from fullwave25_gb300.engine import Engine

    old = os.environ.get("FWGB_VARIANT")
    os.environ["FWGB_VARIANT"] = variant
    try:
        return Engine(inp, validate=False)
    finally:
        if old is None:
            del os.environ["FWGB_VARIANT"]
        else:
            os.environ["FWGB_VARIANT"] = old
