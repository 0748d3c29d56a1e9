// Element stiffness, CSR assembly and boundary integrals (filled in below).
#include "form.hpp"
#include "sfx.h"

using namespace sfx_impl;

extern "C" {
int sfx_form_add_boundary_integral(sfx_form, int, int, const double*) { return fail(SFX_ERR_UNSUPPORTED, "boundary integrals not built yet"); }
int sfx_csr_nnz(sfx_form, int64_t*) { return fail(SFX_ERR_UNSUPPORTED, "assembly not built yet"); }
int sfx_csr_graph(sfx_form, int64_t*, int32_t*, void*) { return fail(SFX_ERR_UNSUPPORTED, "assembly not built yet"); }
int sfx_assemble_csr(sfx_form, double*, void*) { return fail(SFX_ERR_UNSUPPORTED, "assembly not built yet"); }
int sfx_assemble_diagonal(sfx_form, double*, void*) { return fail(SFX_ERR_UNSUPPORTED, "assembly not built yet"); }
}
