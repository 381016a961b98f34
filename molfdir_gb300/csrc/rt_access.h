// rt_access.h -- accessors the host-only translation units (plain C++,
// no CUDA headers) use on the opaque context.
#pragma once

#include "../../include/rotran_gb300.h"

int rt_internal_mfil(rt_ctx* c);
int rt_internal_breit(rt_ctx* c);
int rt_internal_nkr(rt_ctx* c);
int rt_internal_nsc(rt_ctx* c);
int rt_internal_nsc1(rt_ctx* c);
const int* rt_internal_imoras(rt_ctx* c);
void rt_internal_set_error(rt_ctx* c, const char* msg);
// message of rt_last_error(NULL) on the calling thread (context-free calls)
void rt_internal_set_thread_error(const char* msg);
