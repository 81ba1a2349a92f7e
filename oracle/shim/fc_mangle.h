/* Stand-in for the CMake-generated Fortran name-mangling header: maps the
 * BLAS/LAPACK names the reference calls onto the oracle's plain-loop
 * implementations in oracle/shim/blas_shim.cpp (test infrastructure only). */
#ifndef ORACLE_SHIM_FC_MANGLE_H
#define ORACLE_SHIM_FC_MANGLE_H
#define DAXPY oracle_daxpy
#define SAXPY oracle_saxpy
#define DSCAL oracle_dscal
#define SSCAL oracle_sscal
#define DCOPY oracle_dcopy
#define SCOPY oracle_scopy
#define DDOT oracle_ddot
#define SDOT oracle_sdot
#define DNRM2 oracle_dnrm2
#define SNRM2 oracle_snrm2
#define IDAMAX oracle_idamax
#define ISAMAX oracle_isamax
#define DROT oracle_drot
#define SROT oracle_srot
#define DGEMM oracle_dgemm
#define SGEMM oracle_sgemm
#define DGEMV oracle_dgemv
#define SGEMV oracle_sgemv
#define DSYRK oracle_dsyrk
#define SSYRK oracle_ssyrk
#define DTRSM oracle_dtrsm
#define STRSM oracle_strsm
#define DTRMM oracle_dtrmm
#define DSYMV oracle_dsymv
#define DSYMM oracle_dsymm
#define DPOTRF oracle_dpotrf
#define DPOTRS oracle_dpotrs
#define DPOTRI oracle_dpotri
#define DSYEV oracle_dsyev
#define FC_GLOBAL(name, NAME) oracle_##name
#define FC_GLOBAL_(name, NAME) oracle_##name
#endif
