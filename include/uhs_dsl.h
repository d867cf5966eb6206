/*
 * uhs_dsl.h -- reader for UHStencil's stencil DSL (.dsl files).
 *
 * Replaces the front end of the reference's stenCC
 * (UHStencil/include/Parser/Lexer.h, Parser.h:37-606 and
 * lib/Parser/MLIRGen.cpp:183-480) for the purpose the backend needs: turning
 * a stencil program into a uhs_stencil_desc.  The grammar and its quirks
 * follow the reference parser:
 *   - one `stencil NAME(float|double ARG[d]..[d], ...) { ... }` per file;
 *   - body items iteration(T), mpiTile(..), mpiHalo([a,b]..), operation(K),
 *     kernel K { tile(..) swCacheAt(n) domain([lb,ub]..) expr { ... } };
 *   - `+ -` bind at 20 and `* /` at 40, left associative (Parser.h:591-606);
 *   - a leading `-` is allowed on a number only (Parser.h:466-481);
 *   - array indices are positional: in `a[z-1][y][x+2]` the letters are
 *     ignored and the offsets apply to the dimensions in bracket order,
 *     slowest first (Parser.h:527-530);
 *   - an integer index `c[3]` marks a parameter array (Parser.h:551-563);
 *   - `#` starts a comment that runs to the end of the line.
 * The operation kernel's expression is reduced to the linear form
 * sum_k c_k * in[p + o_k]; references to other kernels are inlined
 * (spatial producer -> consumer fusion, the reference's kernel-fusion pass,
 * lib/Dialect/Stencil/StencilKernelFusion.cpp:66-183).
 */
#ifndef UHS_DSL_H_
#define UHS_DSL_H_

#include "uhs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct uhs_program uhs_program; /* opaque, owned by the caller */

/* Parse DSL text.  filename is used in error messages only (may be NULL).
 * On failure returns UHS_EPARSE (or UHS_EUNSUPPORTED for a well-formed
 * program the linear form cannot express) and uhs_last_error() holds
 * "file@line:col: ..." */
int uhs_dsl_parse(const char *text, const char *filename, uhs_program **out);

void uhs_program_free(uhs_program *p);

/* Program name (the `stencil NAME`). */
const char *uhs_program_name(const uhs_program *p);

/* Descriptor of the operation kernel.  desc->terms and desc->params point
 * into storage owned by p.  sizes receives the struct array's extents padded
 * to rank 3 (sizes[0] = 1 for rank 2).  dtype is the program's element type. */
int uhs_program_desc(const uhs_program *p, uhs_stencil_desc *desc, int64_t sizes[3]);

/* 1 when evaluating the linear form left to right rounds exactly like the
 * expression as written (a left-deep sum of coefficient * access terms); 0
 * when the reduction distributed constants or reassociated sums. */
int uhs_program_exact_order(const uhs_program *p);

/* Tile hint of the operation kernel (tile(...) in the DSL), slowest first,
 * zero-padded; returns the number of entries given. */
int uhs_program_tile(const uhs_program *p, int64_t tile[3]);

/* Number of kernels in the program and of parameter arrays. */
int uhs_program_num_kernels(const uhs_program *p);
int uhs_program_num_param_arrays(const uhs_program *p);

/* Set the values of the program's parameter array (the DSL's `c[5]` argument)
 * that coefficient terms index. */
int uhs_program_set_params(uhs_program *p, const double *values, int32_t n);

#ifdef __cplusplus
}
#endif
#endif /* UHS_DSL_H_ */
