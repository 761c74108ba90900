/* Declaration-only stand-in for psrdada's dada_cuda.h (see ipcbuf.h). */
#pragma once
#include "dada_hdu.h"
int dada_cuda_dbregister(dada_hdu_t* hdu);
