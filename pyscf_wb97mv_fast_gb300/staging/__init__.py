"""Staged SCF driver (``schedule.StagedSCF``, ``schedule.run_staged``)."""
