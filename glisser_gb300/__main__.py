"""`python -m glisser_gb300 [--force] [--quiet] [<config>]`: the reference's
command line (targets/main.cpp:29-60, config.in by default) over the C ABI's
glisser_run, which writes everything main() writes under Output-Folder.  A
non-empty output folder is refused unless --force is given (the reference asks
on stdin instead)."""
import argparse
import sys

from . import GlisserError, Simulation, build


def main(argv=None):
    ap = argparse.ArgumentParser(prog="glisser", description="GPU long-term integrator for massless test particles")
    ap.add_argument("config", nargs="?", default="config.in")
    ap.add_argument("--force", action="store_true", help="write into a non-empty output folder")
    ap.add_argument("--quiet", action="store_true", help="do not echo the run log to stdout")
    args = ap.parse_args(argv)
    print("Reading from configuration file %s" % args.config, flush=True)
    try:
        text = open(args.config).read()
    except OSError as e:
        print("Could not read configuration.\n%s" % e, file=sys.stderr)
        return 255
    build()
    try:
        Simulation(text).run(quiet=args.quiet, force=args.force)
    except GlisserError as e:
        print(str(e), file=sys.stderr)
        return 255
    return 0


if __name__ == "__main__":
    sys.exit(main())
