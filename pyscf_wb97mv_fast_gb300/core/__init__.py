"""Subpackage of pyscf_wb97mv_fast_gb300."""
