"""CPU oracle for the catalogue -> SFB coefficient path.  TEST INFRASTRUCTURE.

This package is the oracle the GPU results are tested against, not the
product.  Only the test-suite, the
``smoke()`` check and the ``cpu_baseline`` / ``--impl reference`` legs of the
benchmark import it.  Nothing in the shipped library calls it.

It restates, in FP64 numpy, the reference algorithm of SuperFaB's
``cat2amln`` (``src/cat2anlm.jl:257-310``) and its neighbours:

* ``healpix``   HEALPix RING geometry, ``pix2ang``/``ang2pix`` written from the
                published algorithm (Gorski et al. 2005, ApJ 622, 759), which
                Healpix.jl 4.2.2 implements (reference call sites
                ``src/cat2anlm.jl:230,263``, ``src/windows.jl:198``);
* ``sht``       map2alm / alm2map with uniform 4pi/npix quadrature and the
                ``niter`` Jacobi refinement that Healpix.jl's ``map2alm!``
                applies (reference ``src/healpix_helpers.jl:50-56``);
* ``sfb``       per-(n,l) cubic-spline scatter + SHT (``cat2amln``),
                ``field2anlm_v2``, ``anlm2field`` and ``win_rhat_ln``.

Pinning: the reference ships no golden a_nlm vectors and cannot run here
(no Julia).  The oracle is pinned by the reference's own known-answer tests
(``test/test_cat2anlm.jl``, ``test/test_toplevel.jl``, ``test/test_gnl.jl``,
``test/test_windows.jl``), re-expressed in ``tests/test_oracle_kat.py``, and by
closed-form fixtures in ``tests/golden/``.  Parity is unpinned for the exact
niter=3 result of libsharp at lmax close to 3*nside and for the last-ulp
behaviour of Healpix.jl's ``ang2pixRing``.
"""
