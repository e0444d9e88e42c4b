"""octrecon's command line with the "gb300" device registered.

    python -m oct_recon_af_v1_gb300.octrecon_cli reconstruct <OCTVolume> \\
        --output-root DIR --output-name NAME --set device=\\"gb300\\"

Everything after the module name is octrecon's own CLI (octrecon/cli.py);
octrecon must be importable (installed, or its source folder on PYTHONPATH).
"""
from __future__ import annotations

import sys


def main(argv=None):
    from .plugin import register
    register()
    from octrecon.cli import main as octrecon_main
    return octrecon_main(argv)


if __name__ == "__main__":
    sys.exit(main())
