"""`python -m tapkee_gb300`: the command-line tool (tapkee_gb300.cli)."""
import sys

from .cli import main

sys.exit(main())
