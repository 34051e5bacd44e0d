// Launch arguments of the stepper kernels (host/device shared).
#pragma once

namespace cb {

// XY_FUSED (FP32 form): the sums of XY_REDUCE_FULL and the lambda-free
// nonlinear partials G'', w of the same state in one pass; the penalty terms
// enter in the next z pass, once the sums have given lambda.
enum XYMode { XY_REDUCE_FULL = 0, XY_REDUCE_S = 1, XY_NONLIN = 2, XY_FUSED = 3, XY_INV_PLAIN = 4, XY_FWD_PLAIN = 5 };
// how an xy pass runs (cb_params.xy_split): the size rule (one CTA per plane where two
// fields fit, two-CTA clusters for the FP32 fused pass, else split), the split y/x
// passes, one CTA per plane, or two-CTA clusters for the FP32 fused pass
enum XYPath { XYP_AUTO = 0, XYP_SPLIT = 1, XYP_SINGLE = 2, XYP_CLUSTER = 3 };

struct XYArgs {
    int mode;
    int role;           // partial set and Scal record the pass reads / writes
    int skip_if_stale;  // XY_NONLIN on the state: skip when the stored N_u is reused
    int curv;           // FP32 XY_FUSED with spontaneous curvature: the third output field q
    const void* cin;    // XY_INV_PLAIN: partial C[nz][ny][nc]
    double* rout;       // XY_INV_PLAIN: real double[nz][ny][nx]
    const double* rin;  // XY_FWD_PLAIN: real double[nz][ny][nx]
    void* cout;         // XY_FWD_PLAIN: partial C[nz][ny][nc]
};

enum ZMode {
    Z_ETD2_S1 = 0,  // N_u (fresh) ; a-hat = e phi-hat + c1 N_u                     (Calc.cu:446-457)
    Z_ETD2_S2,      // phi-hat' = a-hat + c2 (N_a - N_u)                           (Calc.cu:466-479)
    Z_ETD4_S1,      // N_u ; a-hat = e_h phi-hat + c_h N_u                          (Calc.cu:488-499)
    Z_ETD4_S2,      // N_a ; b-hat = e_h phi-hat + c_h N_a                          (Calc.cu:509-520)
    Z_ETD4_S3,      // N_b ; c-hat = e_h a-hat + c_h (2 N_b - N_u)                  (Calc.cu:529-540)
    Z_ETD4_S4,      // phi-hat' = e2 phi-hat + f1 N1 + f2 (N1 + N_b) + f3 N_c      (Calc.cu:549-569)
    Z_EULER,        // phi-hat' = phi-hat - dt ga R-hat                             (Calc.cu:393-402)
    Z_INV_STATE,    // partials + Parseval of an existing spectrum (set-up / restore)
    Z_FWD_PLAIN,    // partial -> spectrum (x 1/N)
    Z_INV_PLAIN,    // spectrum (x multiplier) -> partial P0
};

// y-column pass of the split plane path (split_kernels.cuh)
enum YMode { Y_INV2 = 0, Y_INV1, Y_FWD2, Y_FWD1 };

struct YArgs {
    int mode;
    int role;           // stepping: partial set read (inverse)
    int stepping;       // 1: instance buffers (P / Y / A, B) and the done / stale checks
    int skip_if_stale;
    int fused;          // forward of an XY_FUSED pass: outputs go to the role's slot
    int pad;
    const void* cin;    // plain inverse: partial C[nz][ny][nc]
    void* cout;         // plain forward: partial C[nz][ny][nc]
};

enum SpecMul { SM_NONE = 0, SM_LAP = 1, SM_DX = 2, SM_DY = 3, SM_DZ = 4 };

// state_io bits for the plain z modes: the spectrum read (1) or written (2) is
// a stepped state field (double-float pairs in the FP32 form); in the FP64 pass,
// the spectrum read (4) or written (8) is the FP32 form's state, as double-float
// pairs (hi.x, hi.y, lo.x, lo.y) with hi = fl32(v), lo = fl32(v - hi)
enum { IO_CIN_STATE = 1, IO_COUT_STATE = 2, IO_CIN_FF = 4, IO_COUT_FF = 8 };

struct ZArgs {
    int mode;
    int role;      // partial set / Scal record written (stage modes), spectrum read (Z_INV_STATE)
    int mul;       // SpecMul for Z_INV_PLAIN
    int state_io;  // IO_* bits (Z_FWD_PLAIN / Z_INV_PLAIN)
    int curv;      // FP32 stage modes with spontaneous curvature: the third partial q
    int pad;
    const void* cin;
    void* cout;
};

}  // namespace cb
