/* header_c.c - include/pfgpu.h compiled as C99 (tests/test_cabi.py): the
   boundary is a C ABI, so the header must stand alone in a C translation
   unit and name every entry point with C linkage. */
#include "pfgpu.h"

int pfg_header_c_check(void) {
    pfg_options o;
    pfg_default_options(&o);
    pfg_resolve_options(&o);
    size_t a, b, c;
    pfg_abi_sizes(&a, &b, &c);
    return (int)(a == sizeof(pfg_options) && b == sizeof(pfg_stats) && c == sizeof(pfg_result_sizes));
}
