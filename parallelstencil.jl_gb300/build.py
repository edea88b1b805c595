"""Build libps_b200.so in-tree: ``python parallelstencil.jl_gb300/build.py [--force]``."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from ps_gb300._build import main  # noqa: E402

if __name__ == "__main__":
    sys.exit(main())
