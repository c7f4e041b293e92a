// Included by the reference predictor sources but not used by them.
#ifndef LMC_ORACLE_SHIM_BOOST_RANGE_COMBINE_
#define LMC_ORACLE_SHIM_BOOST_RANGE_COMBINE_
#endif
