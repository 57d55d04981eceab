/* Test-only stand-in: utils/set_cosmo_dist.c includes GSL's integration header but calls nothing
 * from it, so an empty header lets oracle/build_ref.py compile that file unchanged. */
#ifndef CF_GSL_SHIM_INTEGRATION_H
#define CF_GSL_SHIM_INTEGRATION_H
#endif
