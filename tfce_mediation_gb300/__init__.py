"""GB300-native permutation-inference path of TFCE_mediation.

Drop-in modules for the reference's operator API (``tfce``, ``cynumstats``,
``pyfunc``, ``tm_func``) backed by hand-written sm_103a CUDA kernels through
the C-ABI in ``include/tfce_gb300.h``:

* ``engine``    -- batched permutation engines (GLM / F / cosinor maps, mediation)
* ``rm_anova``  -- repeated-measures ANCOVA engine (tm-models)
* ``randomise`` -- drop-ins for the reference's permutation drivers
* ``fwer``      -- 1-p(FWER) maps; ``shard`` -- replicas over permutation ranges
* ``gd_fwhm``   -- geodesic FWHM smoothing; ``tmi`` -- TMI container I/O
* ``tail``      -- learned GPD tail of the max-TFCE null
"""
__version__ = "0.1.0"
