"""``python -m lucivant_sim_gb300``: the command-line front end (:mod:`lucivant_sim_gb300.cli`)."""

from lucivant_sim_gb300.cli import main

raise SystemExit(main())
