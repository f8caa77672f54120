"""python -m acvd_gb300.acvd file nvertices gradation [options]  (the reference's ACVD program)."""
import sys

from .cli import main_acvd

if __name__ == "__main__":
    sys.exit(main_acvd())
