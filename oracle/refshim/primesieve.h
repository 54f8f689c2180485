/* primesieve C header stand-in: only the version macro the reference prints. */
#ifndef CTD_REFSHIM_PRIMESIEVE_H
#define CTD_REFSHIM_PRIMESIEVE_H
#define PRIMESIEVE_VERSION "oracle-shim"
#endif
