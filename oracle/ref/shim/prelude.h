// Included before every reference header of the oracle's reference build (g++ -include):
// the LAPACK routines that core/utility/blitzlapack.h declares as <name>_ are the ones in
// the LAPACK that ships inside scipy, exported as scipy_<name>_. Test infrastructure only.
#ifndef ORACLE_REF_PRELUDE_H
#define ORACLE_REF_PRELUDE_H
#define zgbsv_ scipy_zgbsv_
#define zgbtrf_ scipy_zgbtrf_
#define zgbtrs_ scipy_zgbtrs_
#define zgeev_ scipy_zgeev_
#define zgels_ scipy_zgels_
#define zgeqrf_ scipy_zgeqrf_
#define zgetrf_ scipy_zgetrf_
#define zgetri_ scipy_zgetri_
#define zgetrs_ scipy_zgetrs_
#define zhbgv_ scipy_zhbgv_
#define zheev_ scipy_zheev_
#define zpbsvx_ scipy_zpbsvx_
#define zpbtrf_ scipy_zpbtrf_
#define zpbtrs_ scipy_zpbtrs_
#define zungqr_ scipy_zungqr_
#define zunmqr_ scipy_zunmqr_
#endif
