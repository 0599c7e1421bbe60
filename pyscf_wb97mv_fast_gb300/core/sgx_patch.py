"""Fix of the range-separated branch of PySCF 2.14's ``SGX.get_jk``
(reference: pyscf_wb97mv_fast/core/sgx_patch.py:1-63).

Stock PySCF handles ``get_jk(..., omega=w)`` by making a shallow copy of the
SGX object per omega and calling its ``get_jk`` positionally, which has two
effects that this patch removes:

* the positional call leaves out ``vhfopt``, so ``with_j``/``with_k`` and
  ``direct_scf_tol`` land one slot off: an attenuated J is built and thrown
  away on every long-range K, and the caller's ``direct_scf_tol`` is lost;
* the shallow copy shares ``_pjs_data`` (the screening bounds of the full
  1/r kernel) with its parent, so the long-range build is screened with the
  wrong bounds.

``apply()`` replaces ``SGX.get_jk`` by a version whose omega branch keeps the
per-omega copies in ``self._rsh_df`` under PySCF's own key ``'%.6f' % omega``
(the COSX hook recognises those copies), clears the copy's cached
screening/J state, and forwards every argument by keyword under
``mol.with_range_coulomb(omega)``.  The full-range call (omega None) is the
stock one.  ``revert()`` puts the stock method back.  Importing this module
does not import PySCF; ``apply`` does.
"""

_state = {'module': None, 'orig': None}


def _sgx_module():
    import pyscf.sgx.sgx as mod
    return mod


def _rsh_copy(sgx, key):
    """The per-omega SGX copy of sgx, created on first use."""
    table = sgx._rsh_df
    rsh = table.get(key)
    if rsh is None:
        rsh = sgx.copy()
        # no nested copies, and nothing cached for the full 1/r kernel
        rsh._rsh_df = None
        rsh._vjopt = None
        rsh._overlap_correction_matrix = None
        rsh._pjs_data = None
        table[key] = rsh
    return rsh


def make_get_jk(orig):
    """The patched SGX.get_jk around the stock method orig."""
    def get_jk(self, dm, hermi=1, vhfopt=None, with_j=True, with_k=True,
               direct_scf_tol=1e-13, omega=None):
        if omega is None:
            return orig(self, dm, hermi, vhfopt, with_j, with_k,
                        direct_scf_tol)
        rsh = _rsh_copy(self, '%.6f' % omega)
        with rsh.mol.with_range_coulomb(omega):
            return orig(rsh, dm, hermi, vhfopt=vhfopt, with_j=with_j,
                        with_k=with_k, direct_scf_tol=direct_scf_tol)
    get_jk._wb_sgx_patch = True
    return get_jk


def apply(module=None):
    """Install the fix on module.SGX (default pyscf.sgx.sgx).  Idempotent."""
    mod = module if module is not None else _sgx_module()
    cur = mod.SGX.get_jk
    if getattr(cur, '_wb_sgx_patch', False):
        return
    _state['module'], _state['orig'] = mod, cur
    mod.SGX.get_jk = make_get_jk(cur)


def revert():
    """Put the stock SGX.get_jk back (no-op when not applied)."""
    mod, orig = _state['module'], _state['orig']
    if mod is None:
        return
    mod.SGX.get_jk = orig
    _state['module'] = _state['orig'] = None


def applied():
    return _state['module'] is not None
