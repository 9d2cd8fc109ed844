/* Stand-in for gsl_sf_legendre_Pl (Bonnet recurrence).  Test infrastructure. */
#ifndef AAR_SHIM_GSL_LEGENDRE_H
#define AAR_SHIM_GSL_LEGENDRE_H
double gsl_sf_legendre_Pl(int l, double x);
#endif
