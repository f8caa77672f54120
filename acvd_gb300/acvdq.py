"""python -m acvd_gb300.acvdq file nvertices gradation [options]  (the reference's ACVDQ program)."""
import sys

from .cli import main_acvdq

if __name__ == "__main__":
    sys.exit(main_acvdq())
