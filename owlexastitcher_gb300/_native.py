"""Locates the in-tree native libraries.  There is no fallback: a missing
library is an error that names the build step."""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))


def lib_path(name):
    p = os.path.join(PKG_DIR, name)
    if not os.path.exists(p):
        raise RuntimeError(
            f"{name} is not built ({p} missing); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python -m owlexastitcher_gb300.build`")
    return p
