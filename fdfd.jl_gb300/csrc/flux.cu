// Field post-processing: Poynting flux and its line integral (src/flux.jl).
//
//   poynting (flux.jl:15-29), per cell, with grid_average(a, w) = (a + a shifted
//   by one cell along w)/2 (periodic, grid.jl:157-162):
//     TM: Sx = -½ Re(avgx(Ez)·conj(Hy)),  Sy = ½ Re(avgy(Ez)·conj(Hx))
//     TE: Sx =  ½ Re(Ey·conj(avgx(Hz))),  Sy = -½ Re(Ex·conj(avgy(Hz)))
//   (the reference's TE branch reads `field.Hz_x`/`field.Hz_y`, fields a FieldTE
//   does not have; the averaged Hz it has just computed is meant and used here).
//
//   flux_surface_integral with an x̂ normal (flux.jl:37-57): at column xind, over
//   the rows iy0..iy1,
//     TM: Σ -½ Re(½(Ez[xind] + Ez[xind+1])·conj(Hy[xind]))·dy
//     TE: Σ -½ Re(Ey[xind]·conj(½(Hz[xind] + Hz[xind+1])))·dy
//   (the reference's TE branch names an undefined `pt` and reads :Hy; the column
//   of `center` and :Ey are meant and used here; the sign is the reference's).
//
// Fields are FP64 complex, natural order (x fastest), f1/f2/f3 = (Ez, Hx, Hy) for
// TM or (Hz, Ex, Ey) for TE.
#include "common.cuh"
#include "kernels.cuh"

__global__ void poynting_kernel(int Nx, int Ny, int pol, const cplx<double>* __restrict__ f1,
                                const cplx<double>* __restrict__ f2, const cplx<double>* __restrict__ f3,
                                double* __restrict__ Sx, double* __restrict__ Sy) {
    const long long N = (long long)Nx * Ny;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int ix = (int)(k % Nx), iy = (int)(k / Nx);
    const long long kxm = ix == 0 ? k + Nx - 1 : k - 1;
    const long long kym = iy == 0 ? k + N - Nx : k - Nx;
    const cplx<double> a = f1[k];
    const cplx<double> ax = cscale(cadd(a, f1[kxm]), 0.5), ay = cscale(cadd(a, f1[kym]), 0.5);
    // Re(u·conj(v)) = u.re v.re + u.im v.im
    if (pol == 1) {
        const cplx<double> hx = f2[k], hy = f3[k];
        Sx[k] = -0.5 * (ax.re * hy.re + ax.im * hy.im);
        Sy[k] = 0.5 * (ay.re * hx.re + ay.im * hx.im);
    } else {
        const cplx<double> ex = f2[k], ey = f3[k];
        Sx[k] = 0.5 * (ey.re * ax.re + ey.im * ax.im);
        Sy[k] = -0.5 * (ex.re * ay.re + ex.im * ay.im);
    }
}

// One block per line: out[l] = the x̂-normal line integral of line l.  Lines
// are (xind, iy0, iy1) with xind + 1 < Nx checked by the host.
__global__ void flux_line_kernel(int Nx, int pol, double dy, const int3* __restrict__ lines,
                                 const cplx<double>* __restrict__ f1, const cplx<double>* __restrict__ f3,
                                 double* __restrict__ out) {
    const int3 L = lines[blockIdx.x];
    double acc = 0.0;
    for (int iy = L.y + (int)threadIdx.x; iy <= L.z; iy += blockDim.x) {
        const long long k = L.x + (long long)Nx * iy;
        const cplx<double> av = cscale(cadd(f1[k], f1[k + 1]), 0.5);
        const cplx<double> g = f3[k];   // Hy (TM) or Ey (TE)
        acc += -0.5 * (av.re * g.re + av.im * g.im);
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[blockIdx.x] = acc * dy;
    }
    (void)pol;   // Re(Ez̄·conj(Hy)) and Re(Ey·conj(H̄z)) are the same real product
}

void launch_poynting(cudaStream_t s, int Nx, int Ny, int pol, const cplx<double>* f1, const cplx<double>* f2,
                     const cplx<double>* f3, double* Sx, double* Sy) {
    const long long N = (long long)Nx * Ny;
    poynting_kernel<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(Nx, Ny, pol, f1, f2, f3, Sx, Sy);
}

void launch_flux_lines(cudaStream_t s, int nlines, int Nx, int pol, double dy, const int3* lines,
                       const cplx<double>* f1, const cplx<double>* f3, double* out) {
    flux_line_kernel<<<nlines, 256, 0, s>>>(Nx, pol, dy, lines, f1, f3, out);
}
