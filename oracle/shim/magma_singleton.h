/* Empty stand-in: the oracle's pinning build has no MAGMA. */
#ifndef ORACLE_SHIM_MAGMA_SINGLETON_H
#define ORACLE_SHIM_MAGMA_SINGLETON_H
#endif
