/*
 * gmgs_mex.c - MATLAB MEX binding of libgmgs: the reference's solve and
 * stress recovery on one GB300, called from MATLAB with the reference's
 * globals as arguments.
 *
 *   [U, stress, iters, relres] = gmgs_mex(voxelizedVolume_, fixingCond_, loadingCond_, ...
 *                                          tol_, maxIT_, weightFactorJacobi_ [, eleSize [, precision]])
 *
 * replaces GetDeformation() (src/kernel/GetDeformation.m:1-22) and, when a
 * second output is requested, GetCartesianStress() (src/kernel/GetCartesianStress.m:1-42)
 * in src/Demo.m:74-77 and src/GMGS3D.m:29-32:
 *
 *   U_ = gmgs_mex(voxelizedVolume_, fixingCond_, loadingCond_, tol_, maxIT_, weightFactorJacobi_);
 *
 * Inputs
 *   voxelizedVolume_    ny x nx x nz int32 or double, 1 = solid (column-major, as in the reference)
 *   fixingCond_         vector of 1-based compact node ids (all three DOFs fixed)
 *   loadingCond_        n x 4 [id fx fy fz]; a later duplicate id wins
 *   tol_, maxIT_, weightFactorJacobi_   CG tolerance, iteration limit, Jacobi weight
 *   eleSize             optional 1 x 3 voxel edge lengths (x, y, z), default [1 1 1]
 *   precision           optional 0 = FP64 (default, the drop-in), 1 = mixed FP32 V-cycle
 * Outputs
 *   U       3*numNodes x 1 interleaved displacements (U_)
 *   stress  numNodes x 6 nodal stress [xx yy zz yz zx xy] (cartesianStressField_)
 *   iters, relres
 *
 * Build (MATLAB R2018a or later; libgmgs.so built by gmgs-3d_gb300/build.py):
 *   mex gmgs_mex.c -I<repo>/include -L<repo>/gmgs-3d_gb300/gmgs -lgmgs
 * A non-converged solve returns U with a warning, like CG_solver.m:52-55.
 */
#include <stdint.h>
#include <string.h>

#include "gmgs.h"
#include "mex.h"

static void fail(gmgs_handle* h, const char* id, int status) {
    const char* msg = gmgs_last_error(h);
    char buf[512];
    /* copy before the handle goes away */
    strncpy(buf, msg ? msg : gmgs_status_string(status), sizeof(buf) - 1);
    buf[sizeof(buf) - 1] = '\0';
    if (h) gmgs_destroy(h);
    mexErrMsgIdAndTxt(id, "%s (status %d)", buf, status);
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    if (nrhs < 6 || nrhs > 8) mexErrMsgIdAndTxt("gmgs:args", "gmgs_mex needs 6 to 8 arguments");
    if (mxGetNumberOfDimensions(prhs[0]) != 3) mexErrMsgIdAndTxt("gmgs:args", "voxelizedVolume_ must be 3-D");
    if (mxGetN(prhs[2]) != 4) mexErrMsgIdAndTxt("gmgs:args", "loadingCond_ must have 4 columns");
    const mwSize* d = mxGetDimensions(prhs[0]);
    const mwSize nvox = d[0] * d[1] * d[2];

    /* occupancy as int32, column-major (y fastest) */
    int32_t* occ = (int32_t*)mxMalloc(nvox * sizeof(int32_t));
    if (mxIsInt32(prhs[0])) {
        memcpy(occ, mxGetData(prhs[0]), nvox * sizeof(int32_t));
    } else if (mxIsDouble(prhs[0])) {
        const double* v = mxGetPr(prhs[0]);
        for (mwSize i = 0; i < nvox; ++i) occ[i] = (int32_t)v[i];
    } else {
        mexErrMsgIdAndTxt("gmgs:args", "voxelizedVolume_ must be int32 or double");
    }

    gmgs_params p;
    gmgs_default_params(&p);
    p.tol = mxGetScalar(prhs[3]);
    p.max_it = (int32_t)mxGetScalar(prhs[4]);
    p.omega = mxGetScalar(prhs[5]);
    double ele[3] = {1.0, 1.0, 1.0};
    if (nrhs > 6 && mxGetNumberOfElements(prhs[6]) == 3) memcpy(ele, mxGetPr(prhs[6]), sizeof(ele));
    if (nrhs > 7) p.precision = (int32_t)mxGetScalar(prhs[7]);

    gmgs_handle* h = NULL;
    int st = gmgs_create(occ, (int32_t)d[0], (int32_t)d[1], (int32_t)d[2], ele, &p, &h);
    mxFree(occ);
    if (st != GMGS_OK) fail(NULL, "gmgs:create", st);

    /* fixingCond_ arrives as doubles, loadingCond_ as n x 4 column-major: rows for the C ABI */
    const mwSize nf = mxGetNumberOfElements(prhs[1]), nl = mxGetM(prhs[2]);
    int32_t* fx = (int32_t*)mxMalloc((nf ? nf : 1) * sizeof(int32_t));
    double* ld = (double*)mxMalloc((nl ? 4 * nl : 4) * sizeof(double));
    const double* fp = mxGetPr(prhs[1]);
    const double* lp = mxGetPr(prhs[2]);
    for (mwSize i = 0; i < nf; ++i) fx[i] = (int32_t)fp[i];
    for (mwSize i = 0; i < nl; ++i)
        for (int k = 0; k < 4; ++k) ld[4 * i + k] = lp[i + (mwSize)k * nl];
    st = gmgs_set_bc(h, fx, (int64_t)nf, ld, (int64_t)nl);
    mxFree(fx);
    mxFree(ld);
    if (st != GMGS_OK) fail(h, "gmgs:boundary", st);

    int64_t nn = 0;
    gmgs_num_nodes(h, 1, &nn);
    plhs[0] = mxCreateDoubleMatrix((mwSize)(3 * nn), 1, mxREAL);
    int32_t iters = 0;
    double relres = 0.0;
    st = gmgs_solve(h, mxGetPr(plhs[0]), &iters, &relres, NULL);
    if (st == GMGS_ERR_MAX_ITERATIONS)
        mexWarnMsgIdAndTxt("gmgs:maxit", "Exceed the maximum iterate numbers (relative residual %g)", relres);
    else if (st != GMGS_OK)
        fail(h, "gmgs:solve", st);
    if (nlhs > 1) {
        /* gmgs_stress writes nn rows of 6 (row-major); MATLAB wants nn x 6 column-major */
        double* rows = (double*)mxMalloc((size_t)nn * 6 * sizeof(double));
        st = gmgs_stress(h, rows, NULL);
        if (st != GMGS_OK) {
            mxFree(rows);
            fail(h, "gmgs:stress", st);
        }
        plhs[1] = mxCreateDoubleMatrix((mwSize)nn, 6, mxREAL);
        double* out = mxGetPr(plhs[1]);
        for (int64_t i = 0; i < nn; ++i)
            for (int k = 0; k < 6; ++k) out[i + (int64_t)k * nn] = rows[6 * i + k];
        mxFree(rows);
    }
    if (nlhs > 2) plhs[2] = mxCreateDoubleScalar((double)iters);
    if (nlhs > 3) plhs[3] = mxCreateDoubleScalar(relres);
    gmgs_destroy(h);
}
