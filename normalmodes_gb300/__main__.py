"""python -m normalmodes_gb300 global_conf ...: the job driver (run.py)."""
import sys

from .run import main

sys.exit(main())
