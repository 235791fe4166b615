"""Location of the reference checkout for the fixture generators in this folder: the first
command-line argument, else the GTRAP_REFERENCE environment variable."""
import os
import sys
from pathlib import Path


def reference_dir() -> Path:
    path = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GTRAP_REFERENCE")
    if not path or not Path(path).is_dir():
        sys.exit("give the reference checkout as the first argument or in GTRAP_REFERENCE")
    return Path(path)
