"""Recipe modules: ConvectionConfig -> (builder, class, constructor kwargs).

One module per implemented ``viscosity_model``, following the convention of
``specmc/models/const.py:30-57`` (``NAME`` / ``CLS`` / ``BUILDER`` / ``kwargs``
/ ``build`` / ``spec``); ``specmc_gb300.api`` dispatches through them.
"""
