// Internal launcher declarations shared by the library's translation units.
#pragma once
#include <vector>
#include "common.cuh"

// legendre_simt.cu
cudaError_t launch_inv_legendre_simt(const ShtGeom& g, const InvSet& s, bool vec, bool fp64,
                                     cudaStream_t st);
cudaError_t launch_fwd_legendre_simt(const ShtGeom& g, const FwdSet& s, bool vec, bool fp64,
                                     cudaStream_t st);

// fft.cu
// Inverse: half spectrum T2 [n_m][n_theta] -> double grid [n_phi][ld].
// Forward: double grid -> ES/EA half spectrum T2 [n_m][nh][2] (scaled 1/n_phi).
// rows: theta rows per CTA of the fast path (8 or 16; 0 = chosen by size)
// arith: FFT_ARITH_F32 / _F64 / _DF (double-float, working type dfl)
cudaError_t launch_fft_inverse(const ShtGeom& g, const FftSet& s, int arith, int rows, cudaStream_t st);
// the double-float fast path's twiddle tables kept in device memory (ShtGeom::twr) for
// this row length, from the table e^{+2 pi i k / n_phi}; empty when the path keeps them
// in shared memory
std::vector<float4> fft_df_global_twiddles(int n_phi, const std::vector<float4>& twdf);
cudaError_t launch_fft_forward(const ShtGeom& g, const FftSet& s, int arith, int rows, cudaStream_t st);
bool fft_fast_path(int n_phi);

// tables.cu
cudaError_t build_tables_fp64(int l_max, int m_max, int minc, int n_theta, const int* d_lmoff,
                              double* d_theta, double* d_gauss, double* d_P, double* d_dP,
                              double* d_wgt, double* d_osin2, cudaStream_t st);
cudaError_t convert_tables_fp32(const double* P, const double* dP, float* P32, float* dP32,
                                size_t n, cudaStream_t st);

// peak.cu
cudaError_t launch_fma_peak(void* out, bool fp64, int blocks, int iters, cudaStream_t st);

// legendre_tc.cu
cudaError_t launch_wait_selftest(long long max_cycles, int arrive, int* err, cudaStream_t st);
cudaError_t launch_tc_selftest(int n, int kchunks, bool tf32, const float* A, const float* B, float* D, int* err,
                               cudaStream_t st);
void tc_table_layout(const ShtGeom& g, bool tf32, int* ntt, int* nlt, int* ncj, std::vector<long long>& inv_blk0,
                     std::vector<long long>& fwd_blk0, long long* inv_blocks, long long* fwd_blocks);
// the same with `bpc` 16 KB blocks per K chunk
void tc_table_layout_bpc(const ShtGeom& g, int bpc, int* ntt, int* nlt, int* ncj, std::vector<long long>& inv_blk0,
                         std::vector<long long>& fwd_blk0, long long* inv_blocks, long long* fwd_blocks);
cudaError_t build_tc_images(const ShtGeom& g, const TcTables& t, bool tf32, unsigned char* inv_img, float* inv_scale,
                            unsigned char* fwd_img, float* fwd_scale, cudaStream_t st);
cudaError_t launch_inv_legendre_tc(const ShtGeom& g, const InvSet& s, bool vec, const TcTables& t,
                                   cudaStream_t st);
cudaError_t launch_fwd_legendre_tc(const ShtGeom& g, const FwdSet& s, bool vec, const TcTables& t,
                                   cudaStream_t st);
// legendre_tcp.cu (pack kernels + persistent, warp-specialized tensor-core kernels)
// tf32: the 2 x TF32 split form (kind::tf32) instead of 3 x BF16
size_t tcp_data_bytes(const ShtGeom& g, const TcTables& t, int ncplx, bool vec, bool inverse, bool tf32);
cudaError_t launch_inv_legendre_tcp(const ShtGeom& g, const InvSet& s, bool vec, bool tf32, const TcTables& t,
                                    unsigned char* bimg, cudaStream_t st);
cudaError_t launch_fwd_legendre_tcp(const ShtGeom& g, const FwdSet& s, bool vec, bool tf32, const TcTables& t,
                                    unsigned char* bimg, cudaStream_t st);

// nl.cu
cudaError_t launch_get_nl(const ShtGeom& g, const NlGrids& in, const NlGrids& out, const double* or2,
                          double or2_0, int nlev, int arith, cudaStream_t st);

// the general get_nl with the reference's switches; cosn2[nh] = cos/sin^2 of the northern colatitudes
cudaError_t build_cosn2(const ShtGeom& g, const double* theta, double* cosn2, cudaStream_t st);
cudaError_t launch_get_nl_full(const ShtGeom& g, const NlFull& a, const double* cosn2, int nlev, int arith,
                               cudaStream_t st);

// td.cu
cudaError_t launch_get_td(const ShtGeom& g, const TdArgs& a, int nlev, int arith, cudaStream_t st);
cudaError_t build_td_coef(const ShtGeom& g, double2* coef, int* lq, cudaStream_t st);
cudaError_t launch_get_td_full(const ShtGeom& g, const TdFull& a, int nlev, int arith, cudaStream_t st);
// boundary pieces of the radial loop, one level (bcs.cu); theta = the n_theta
// Gauss colatitudes north to south
cudaError_t launch_v_rigid_boundary(const ShtGeom& g, const double* theta, const BcGrids& a, double r2rho0,
                                    double omega, int keep_vr, cudaStream_t st);
cudaError_t launch_v_center_sphere(const ShtGeom& g, const double* theta, const double2* ddw, int lm11, double* vr,
                                   double* vt, double* vp, cudaStream_t st);
cudaError_t launch_br_v_products(const ShtGeom& g, const double* theta, const double* br, const double* vt,
                                 const double* vp, double fac, double omega, double* out_t, double* out_p,
                                 cudaStream_t st);
cudaError_t launch_b_nl_bcs(int K, double fac, const double2* y, double2* x, cudaStream_t st);
int lorentz_torque_blocks(const ShtGeom& g);
cudaError_t launch_lorentz_torque(const ShtGeom& g, const double* theta, const double* br, const double* bp,
                                  double LFfac, double b0, double* partial, double* out, cudaStream_t st);
// per-level maxima into mx[2 * nlev] (zeroed here), then dtrkc / dthkc updated in place
cudaError_t launch_courant(const ShtGeom& g, const CourantArgs& a, int nlev, unsigned long long* mx, double* dtrkc,
                           double* dthkc, cudaStream_t st);

// legendre_oz.cu: the fixed-point tensor-core forms (seven (FP64TC) or five
// (BF16X5) BF16 digits per operand, TcTables::ndig, exact FP32 accumulation);
// TcTables with inv_exp / fwd_exp
void oz_table_layout(const ShtGeom& g, int digits, int* ntt, int* nlt, int* ncj, std::vector<long long>& inv_blk0,
                     std::vector<long long>& fwd_blk0, long long* inv_blocks, long long* fwd_blocks);
cudaError_t build_oz_images(const ShtGeom& g, const TcTables& t, unsigned char* inv_img, short* inv_exp,
                            unsigned char* fwd_img, short* fwd_exp, cudaStream_t st);
// data images (digits + column exponents) of one call of ncplx complex columns
size_t oz_data_bytes(const ShtGeom& g, const TcTables& t, int ncplx, bool inverse);
// synthesis: double-float half spectra in the parity-separated layout of the
// tensor-core forms; analysis: double-float (ES, EA) half spectra in
cudaError_t launch_inv_legendre_oz(const ShtGeom& g, const InvSet& s, bool vec, const TcTables& t,
                                   unsigned char* bimg, cudaStream_t st);
cudaError_t launch_fwd_legendre_oz(const ShtGeom& g, const FwdSet& s, bool vec, const TcTables& t,
                                   unsigned char* bimg, cudaStream_t st);
// several instances in one pack + one persistent launch (magic_sht_group_*):
// oz_layout_insts fills nct, cexp, tile0 and blk0 of every instance (g, s, t
// and bimg set by the caller) and returns the launch's pack blocks and tiles;
// inst[0..n) on the host, d_inst the same array in device memory, n at most
// kMaxGroupInst
template <class Set>
void oz_layout_insts(LegInst<Set>* inst, int n, bool vec, long long* nblocks, long long* ntiles);
cudaError_t launch_inv_legendre_oz_multi(const LegInst<InvSet>* inst, const LegInst<InvSet>* d_inst, int n,
                                         bool vec, long long nblocks, long long ntiles, cudaStream_t st);
cudaError_t launch_fwd_legendre_oz_multi(const LegInst<FwdSet>* inst, const LegInst<FwdSet>* d_inst, int n,
                                         bool vec, long long nblocks, long long ntiles, cudaStream_t st);
// the same for the 3xBF16 persistent kernels (legendre_tcp.cu); cexp unused
template <class Set>
void tcp_layout_insts(LegInst<Set>* inst, int n, bool vec, long long* nblocks, long long* ntiles);
cudaError_t launch_inv_legendre_tcp_multi(const LegInst<InvSet>* inst, const LegInst<InvSet>* d_inst, int n,
                                          bool vec, long long nblocks, long long ntiles, cudaStream_t st);
cudaError_t launch_fwd_legendre_tcp_multi(const LegInst<FwdSet>* inst, const LegInst<FwdSet>* d_inst, int n,
                                          bool vec, long long nblocks, long long ntiles, cudaStream_t st);
