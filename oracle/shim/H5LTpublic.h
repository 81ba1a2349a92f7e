/* Declaration-only stand-in for <H5LTpublic.h> (see hdf5.h shim). */
#ifndef ORACLE_SHIM_H5LTPUBLIC_H
#define ORACLE_SHIM_H5LTPUBLIC_H
#include "hdf5.h"
static inline herr_t H5LTfind_dataset(hid_t, const char*) { return (herr_t)oracle_h5_abort(); }
#endif
