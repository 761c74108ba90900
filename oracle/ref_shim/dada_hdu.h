// Stand-in for psrdada's dada_hdu.h: only key_t is needed by the headers
// compiled here.
#pragma once
#include <sys/types.h>
