"""python -m acvd_gb300.anisotropic_remeshing_q file nvertices gradation [options]  (the reference's
AnisotropicRemeshingQ program)."""
import sys

from .cli import main_anisotropic_remeshing_q

if __name__ == "__main__":
    sys.exit(main_anisotropic_remeshing_q())
