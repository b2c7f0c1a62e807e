"""Drop-in replacements for the reference's forward-model modules.

Put this directory on ``sys.path`` ahead of the reference checkout and the
reference's drivers pick these up unchanged:

    sys.path.insert(0, os.path.dirname(ismc_gb300.dropin.__file__))
    from ISMC import ISMC as pythonISMC          # as Lookup/lookup.py:15-16 does

``ISMC.ISMC`` and ``ISMLMC.ISMLMC`` keep the reference's positional signature
and return value; ``ISMC_ex`` / ``ISMLMC_ex`` additionally take ``seed=`` and
``mode=`` and return (means, standard errors, status).
"""
