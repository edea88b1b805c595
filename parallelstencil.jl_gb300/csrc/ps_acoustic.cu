// ps_acoustic.cu -- acoustic3D (miniapps/acoustic3D.jl:11-21) as one kernel per time step.
//
// The miniapp's step is two `@parallel` launches: compute_V! (`@inn(Vx) = @inn(Vx) -
// dt/ρ*@d_xi(P)/dx`, same for Vy, Vz) and compute_P! (`@all(P) = @all(P) - dt*k*(@d_xa(Vx)/dx +
// @d_ya(Vy)/dy + @d_za(Vz)/dz)`). Run back to back they move 12 words per cell (V read and written,
// P read; V read again, P read and written) against the miniapp's A_eff of 8 (acoustic3D.jl:62).
//
// acoustic_step_kernel does both in one z-sweep. The new P of a cell needs the new velocities on
// its six faces, each a function of the old P on both sides of the face, so a CTA that owns an
// x-y tile computes the faces on its tile's upper edges itself (the neighbour tile computes them
// too, from the same operands, bit for bit). Old and new state live in different arrays (V, P ->
// V2, P2): a CTA reads old values on its neighbours' cells while those neighbours write theirs, so
// an in-place update would race. 8 words per cell: Vx, Vy, Vz, P read once, Vx2, Vy2, Vz2, P2
// written once (every value, faces outside @inn copied).
//
// Thread map: 32 lanes along x; each warp owns K consecutive y rows and sweeps a z range, so the
// new Vy of a face between two of its rows is computed once and used by both cells, the new Vz of
// face z+1 is carried to plane z+1 in registers, and the new Vx of face x+1 comes from lane x+1 by
// a shuffle. Per plane a warp loads its K rows of P(z+1), Vz(z+1), Vx(z), Vy(z), the Vy face and
// the P row just above its rows and the P row below them; lanes 0 and 31 also load the P cell (and
// Vx face) just outside the warp's 32 columns.
//
// Arithmetic: IEEE (FP32 or FP64, the operations and their order of the two-kernel sequence, the
// divisions by dx, dy, dz through div_c: bit-identical to it) or, for FP64 arrays, FP32 pairs
// (ps_dd.cuh): values split on load with integer operations, the constants (dt/ρ)/h and (dt·k)/h
// folded into one product per term (three-float constants), each new value stored as the old
// FP64 value plus the pair increment, summed in FP64.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <utility>

#include "ps_common.cuh"
#include "ps_dd.cuh"

namespace ps {

namespace {

constexpr int ACU_W = 8;  // warps per CTA

template <typename S>
struct AcuArrays {
    const S* __restrict__ Vx;
    const S* __restrict__ Vy;
    const S* __restrict__ Vz;
    const S* __restrict__ P;
    S* __restrict__ Vx2;
    S* __restrict__ Vy2;
    S* __restrict__ Vz2;
    S* __restrict__ P2;
    int64_t nx, ny, nz;
};

// IEEE arithmetic in the storage type: the reference's statements as written (the divisions by
// dx, dy, dz correctly rounded through div_c). The increment form `v + (-x)` equals `v - x`.
template <typename T>
struct AcuIeee {
    using S = T;
    using V = T;
    // CTAs per SM the kernel is compiled for: FP32 fits five (47 registers, no spills), FP64 four
    static constexpr int kMinBlocks = sizeof(T) == 4 ? 5 : 4;
    struct C {
        T dtr, dtk;
        DivC<T> h[3];
    };
    static __device__ __forceinline__ V in(S x, bool&) { return x; }
    static __device__ __forceinline__ V add(V a, V b) { return a + b; }
    static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
    // `- dt/ρ*@d_i(P)/h`: dt/ρ is one host value (Julia evaluates dt/ρ first)
    static __device__ __forceinline__ V vdel(V pa, V pb, const C& c, int d) { return -div_c(c.dtr * (pa - pb), c.h[d]); }
    // `- dt*k*(@d_xa(Vx)/dx + @d_ya(Vy)/dy + @d_za(Vz)/dz)`
    static __device__ __forceinline__ V pdel(V ax, V ay, V az, const C& c) {
        return -(c.dtk * ((div_c(ax, c.h[0]) + div_c(ay, c.h[1])) + div_c(az, c.h[2])));
    }
    static __device__ __forceinline__ S store(S, V nv, V) { return nv; }
    static __device__ __forceinline__ V shfl_up(V v) { return __shfl_up_sync(0xFFFFFFFFu, v, 1); }
    static __device__ __forceinline__ V shfl_down(V v) { return __shfl_down_sync(0xFFFFFFFFu, v, 1); }
};

// FP64 arrays, arithmetic on FP32 pairs; each new value is stored as the caller's FP64 value plus
// the pair increment, summed in FP64 (the state keeps its 53 bits; only increments are 47-bit).
struct AcuSplit {
    using S = double;
    using V = dd;
    static constexpr int kMinBlocks = 4;
    struct C {
        dd cv[3];  // (dt/ρ)/h_d as h + l, and its remainder r (h + l + r exact to ~2^-72)
        dd ck[3];  // (dt·k)/h_d
        float cvr[3], ckr[3];
    };
    // a * (c + r): the constant's third term keeps its rounding out of every step (a bias of
    // ~2^-49 per step would otherwise add up coherently over a run)
    static __device__ __forceinline__ V mulc(V a, dd c, float r) {
        const float p = a.h * c.h;
        float e = fmaf(a.h, c.h, -p);
        e = fmaf(a.h, c.l, e);
        e = fmaf(a.l, c.h, e);
        e = fmaf(a.h, r, e);
        return {p, e};
    }
    static __device__ __forceinline__ V in(S x, bool& big) { return dd_split(x, big); }
    static __device__ __forceinline__ V add(V a, V b) { return dd_add(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return dd_sub(a, b); }
    static __device__ __forceinline__ V vdel(V pa, V pb, const C& c, int d) {
        const V m = mulc(dd_sub(pa, pb), c.cv[d], c.cvr[d]);
        return {-m.h, -m.l};
    }
    static __device__ __forceinline__ V pdel(V ax, V ay, V az, const C& c) {
        const V m = dd_add(dd_add(mulc(ax, c.ck[0], c.ckr[0]), mulc(ay, c.ck[1], c.ckr[1])), mulc(az, c.ck[2], c.ckr[2]));
        return {-m.h, -m.l};
    }
    static __device__ __forceinline__ S store(S raw, V, V dl) { return (raw + f32_to_f64(dl.h)) + f32_to_f64(dl.l); }
    static __device__ __forceinline__ V shfl_up(V v) {
        return {__shfl_up_sync(0xFFFFFFFFu, v.h, 1), __shfl_up_sync(0xFFFFFFFFu, v.l, 1)};
    }
    static __device__ __forceinline__ V shfl_down(V v) {
        return {__shfl_down_sync(0xFFFFFFFFu, v.h, 1), __shfl_down_sync(0xFFFFFFFFu, v.l, 1)};
    }
};

// One y row per warp (each Vy face between two rows is computed by both: two rows per warp measured
// slower, their registers cost occupancy). I: the index type of element offsets (int when every
// array has fewer than 2^31 elements). Offsets advance by the plane strides along the sweep.
template <class AR, typename I>
__global__ void __launch_bounds__(32 * ACU_W, AR::kMinBlocks) acoustic_step_kernel(AcuArrays<typename AR::S> a,
                                                                    typename AR::C c, int Lz, int* err) {
    using S = typename AR::S;
    using V = typename AR::V;
    const int lane = threadIdx.x;
    const I nx = (I)a.nx, ny = (I)a.ny, nz = (I)a.nz;
    const I y = (I)blockIdx.y * ACU_W + (I)threadIdx.y;
    if (y >= ny) return;  // whole warps only: no block-wide synchronisation follows
    const I x = (I)blockIdx.x * 32 + lane;
    const I z0 = (I)blockIdx.z * Lz;
    const I z1 = z0 + Lz < nz ? z0 + Lz : nz;
    const bool xv = x < nx;
    const I sP = nx * ny, sX = (nx + 1) * ny, sY = nx * (ny + 1);  // plane strides: P and Vz, Vx, Vy
    // the x-y parts of the @inn masks
    const bool xin = x >= 1 && x <= nx - 2, yin = y >= 1 && y <= ny - 2;
    const bool m_vx = x >= 1 && yin;              // Vx face x (x <= nx - 1 holds)
    const bool m_vx1 = x + 1 <= nx - 1 && yin;    // Vx face x + 1
    const bool m_vy0 = xin && y >= 1;             // Vy face y (y <= ny - 1 holds)
    const bool m_vy1 = xin && y + 1 <= ny - 1;    // Vy face y + 1
    const bool m_vz = xin && yin;
    const bool ld_lo = xv && y >= 1, ld_hi = xv && y + 1 < ny;
    const bool e_lo = lane == 0 && xv && x >= 1;           // loads P(x-1)
    const bool e_p31 = lane == 31 && xv && x + 1 < nx;     // loads P(x+1)
    const bool e_hi = xv && (lane == 31 || x == nx - 1);   // computes the Vx face x + 1 itself
    const bool last_x = x == nx - 1, last_y = y == ny - 1;
    bool big = false;

    I oP = x + nx * y + sP * z0;        // P(x, y, z) and the Vz face below it
    I oX = x + (nx + 1) * y + sX * z0;  // Vx face x
    I oY = x + nx * y + sY * z0;        // Vy face y
    // carried state: P(z) (value and arithmetic form) and the new Vz on face z
    S pr = xv ? a.P[oP] : S(0);
    V pc = AR::in(pr, big);
    V vzc;
    {
        const S vo = xv ? a.Vz[oP] : S(0);
        const bool inner = m_vz && z0 >= 1;
        const S pm = (xv && inner) ? a.P[oP - sP] : S(0);
        vzc = inner ? AR::add(AR::in(vo, big), AR::vdel(pc, AR::in(pm, big), c, 2)) : AR::in(vo, big);
        if (xv && z0 == 0) a.Vz2[oP] = vo;  // face 0 is outside @inn(Vz)
    }

    // every load runs one plane ahead: P(z+1), the Vz face z+1, the Vx and Vy faces of z, the Vy face
    // y+1, the P rows y-1 and y+1 and the edge lanes' P and Vx values of the plane
    const I xe = lane == 0 ? -1 : 1;  // the edge lanes' neighbour column
    S f_pn = (xv && z0 + 1 < nz) ? a.P[oP + sP] : S(0);
    S f_vzo = xv ? a.Vz[oP + sP] : S(0);
    S f_vxo = xv ? a.Vx[oX] : S(0);
    S f_vy0 = xv ? a.Vy[oY] : S(0);
    S f_vy1 = xv ? a.Vy[oY + nx] : S(0);  // face y + 1 <= ny
    S f_plo = ld_lo ? a.P[oP - nx] : S(0);
    S f_phi = ld_hi ? a.P[oP + nx] : S(0);
    S f_xep = (e_lo || e_p31) ? a.P[oP + xe] : S(0);
    S f_xev = e_hi ? a.Vx[oX + 1] : S(0);
    for (I z = z0; z < z1; ++z, oP += sP, oX += sX, oY += sY) {
        const bool zin = z >= 1 && z <= nz - 2;  // the z range of @inn(Vx), @inn(Vy)
        const S pn = f_pn, vzo = f_vzo, vxo = f_vxo, vy0 = f_vy0;
        const S vy1 = f_vy1, plo = f_plo, phi = f_phi, xep = f_xep, xev = f_xev;
        if (z + 1 < z1) {
            f_pn = (xv && z + 2 < nz) ? a.P[oP + 2 * sP] : S(0);
            f_vzo = xv ? a.Vz[oP + 2 * sP] : S(0);  // face z + 2 <= nz
            f_vxo = xv ? a.Vx[oX + sX] : S(0);
            f_vy0 = xv ? a.Vy[oY + sY] : S(0);
            f_vy1 = xv ? a.Vy[oY + sY + nx] : S(0);
            f_plo = ld_lo ? a.P[oP + sP - nx] : S(0);
            f_phi = ld_hi ? a.P[oP + sP + nx] : S(0);
            f_xep = (e_lo || e_p31) ? a.P[oP + sP + xe] : S(0);
            f_xev = e_hi ? a.Vx[oX + sX + 1] : S(0);
        }

        // Vy on faces y and y + 1
        V vyn0 = AR::in(vy0, big), vyn1 = AR::in(vy1, big);
        S st0 = vy0;
        if (m_vy0 && zin) {
            const V dl = AR::vdel(pc, AR::in(plo, big), c, 1);
            vyn0 = AR::add(vyn0, dl);
            st0 = AR::store(vy0, vyn0, dl);
        }
        if (m_vy1 && zin) {
            const V dl = AR::vdel(AR::in(phi, big), pc, c, 1);
            vyn1 = AR::add(vyn1, dl);
            if (last_y) a.Vy2[oY + nx] = AR::store(vy1, vyn1, dl);
        } else if (xv && last_y) {
            a.Vy2[oY + nx] = vy1;  // face ny is outside @inn(Vy)
        }
        // Vx on face x (this lane) and face x + 1 (the next lane, or computed here at the edges)
        V pxm = AR::shfl_up(pc);
        if (lane == 0) pxm = AR::in(xep, big);
        const bool in_x = m_vx && zin;
        const V vxo_v = AR::in(vxo, big);
        const V dlx = AR::vdel(pc, pxm, c, 0);
        const V vxn = in_x ? AR::add(vxo_v, dlx) : vxo_v;
        V vxp = AR::shfl_down(vxn);
        if (e_hi) {
            const V vo1 = AR::in(xev, big);
            vxp = (m_vx1 && zin) ? AR::add(vo1, AR::vdel(AR::in(xep, big), pc, c, 0)) : vo1;
            if (last_x) a.Vx2[oX + 1] = xev;  // face nx is outside @inn(Vx)
        }
        // Vz on face z + 1
        const bool in_z = m_vz && z + 1 <= nz - 1;
        const V vzo_v = AR::in(vzo, big);
        const V pnv = AR::in(pn, big);
        const V dlz = AR::vdel(pnv, pc, c, 2);
        const V vzn = in_z ? AR::add(vzo_v, dlz) : vzo_v;
        // P
        const V dlp = AR::pdel(AR::sub(vxp, vxn), AR::sub(vyn1, vyn0), AR::sub(vzn, vzc), c);
        if (xv) {
            a.Vy2[oY] = st0;
            a.Vx2[oX] = in_x ? AR::store(vxo, vxn, dlx) : vxo;
            a.Vz2[oP + sP] = in_z ? AR::store(vzo, vzn, dlz) : vzo;
            a.P2[oP] = AR::store(pr, AR::add(pc, dlp), dlp);
        }
        vzc = vzn;
        pc = pnv;
        pr = pn;
    }
    if (big) atomicOr(err, DEV_ERR_RANGE);
}

template <class AR, typename I>
int launch_acoustic_i(const ps_array& Vx, const ps_array& Vy, const ps_array& Vz, const ps_array& P, const ps_array& Vx2,
                      const ps_array& Vy2, const ps_array& Vz2, const ps_array& P2, const typename AR::C& c,
                      const DeviceState* st, cudaStream_t s) {
    using S = typename AR::S;
    AcuArrays<S> a{static_cast<const S*>(Vx.ptr), static_cast<const S*>(Vy.ptr), static_cast<const S*>(Vz.ptr),
                   static_cast<const S*>(P.ptr), static_cast<S*>(Vx2.ptr), static_cast<S*>(Vy2.ptr),
                   static_cast<S*>(Vz2.ptr), static_cast<S*>(P2.ptr), P.n[0], P.n[1], P.n[2]};
    const dim3 blk(32, ACU_W, 1);
    const int64_t gx = (a.nx + 31) / 32, gy = (a.ny + ACU_W - 1) / ACU_W;
    if (gx > 0x7FFFFFFF || gy > 65535) return fail(PS_ERR_SHAPE, "ps_acoustic3d_step: grid too large");
    static int slots_per_sm = 0;  // per instantiation
    if (slots_per_sm == 0) slots_per_sm = resident_ctas(acoustic_step_kernel<AR, I>, 32 * ACU_W, 0);
    int Lz = auto_loopsize(gx * gy, a.nz, (int64_t)slots_per_sm * st->num_sms);
    if ((a.nz + Lz - 1) / Lz > 65535) Lz = (int)((a.nz + 65534) / 65535);
    const dim3 grd((unsigned)gx, (unsigned)gy, (unsigned)((a.nz + Lz - 1) / Lz));
    acoustic_step_kernel<AR, I><<<grd, blk, 0, s>>>(a, c, Lz, st->d_err);
    return PS_OK;
}

template <class AR>
int launch_acoustic(const ps_array& Vx, const ps_array& Vy, const ps_array& Vz, const ps_array& P, const ps_array& Vx2,
                    const ps_array& Vy2, const ps_array& Vz2, const ps_array& P2, const typename AR::C& c,
                    const DeviceState* st, cudaStream_t s) {
    // 32-bit element offsets when every offset the kernel forms stays below 2^31 (the largest
    // array, plus a plane of slack for the offsets one plane ahead)
    const int64_t big = std::max(std::max(numel(Vx), numel(Vy)), numel(Vz)) + 2 * (P.n[0] + 1) * (P.n[1] + 1);
    if (big < ((int64_t)1 << 31))
        return launch_acoustic_i<AR, int>(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, c, st, s);
    return launch_acoustic_i<AR, int64_t>(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, c, st, s);
}

// x as h + l + r (three floats); x itself is given as the exact sum hi + lo of two doubles
void split3_host(double hi, double lo, dd* c, float* r) {
    const float h = (float)hi;
    const double rem1 = (hi - (double)h) + lo;
    const float l = (float)rem1;
    const double rem2 = (hi - (double)h - (double)l) + lo;
    *c = {h, l};
    *r = (float)rem2;
}

// q = a / b to ~106 bits as hi + lo (one Newton correction with the exact FMA remainder)
void div2_host(double a, double b, double* hi, double* lo) {
    const double q = a / b;
    const double rem = std::fma(-q, b, a);  // a - q b, exact
    *hi = q;
    *lo = rem / b;
}

int check_acoustic(const ps_array& Vx, const ps_array& Vy, const ps_array& Vz, const ps_array& P,
                   const char* const nm[4]) {  // names of P, Vx, Vy, Vz
    PS_TRY(check_array(P, nm[0]));
    PS_TRY(check_array(Vx, nm[1]));
    PS_TRY(check_array(Vy, nm[2]));
    PS_TRY(check_array(Vz, nm[3]));
    PS_TRY(check_same_dtype(P, Vx, nm[0], nm[1]));
    PS_TRY(check_same_dtype(P, Vy, nm[0], nm[2]));
    PS_TRY(check_same_dtype(P, Vz, nm[0], nm[3]));
    const int64_t nx = P.n[0], ny = P.n[1], nz = P.n[2];
    PS_TRY(check_shape(Vx, nx + 1, ny, nz, nm[1]));
    PS_TRY(check_shape(Vy, nx, ny + 1, nz, nm[2]));
    PS_TRY(check_shape(Vz, nx, ny, nz + 1, nm[3]));
    return PS_OK;
}

const char* const kNames[4] = {"P", "Vx", "Vy", "Vz"};
const char* const kNames2[4] = {"P2", "Vx2", "Vy2", "Vz2"};

bool overlaps(const ps_array& a, const ps_array& b) {
    const char* a0 = static_cast<const char*>(a.ptr);
    const char* b0 = static_cast<const char*>(b.ptr);
    return a0 < b0 + numel(b) * elsize(b.dtype) && b0 < a0 + numel(a) * elsize(a.dtype);
}

int acoustic_step(const ps_array& Vx, const ps_array& Vy, const ps_array& Vz, const ps_array& P, const ps_array& Vx2,
                  const ps_array& Vy2, const ps_array& Vz2, const ps_array& P2, double dt, double rho, double k,
                  double dx, double dy, double dz, int32_t fp64_mode, const DeviceState* st, cudaStream_t s) {
    if (P.dtype == PS_F32) {
        if (fp64_mode != PS_FP64_IEEE) return fail(PS_ERR_UNSUPPORTED, "ps_acoustic3d_step: fp64_mode needs FP64 arrays");
        // FP32: the scalars are FP32 numbers, dt/ρ and dt·k evaluated in FP32 (Float32 Data.Number)
        AcuIeee<float>::C c{(float)dt / (float)rho, (float)dt * (float)k,
                            {make_div((float)dx), make_div((float)dy), make_div((float)dz)}};
        return launch_acoustic<AcuIeee<float>>(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, c, st, s);
    }
    if (fp64_mode == PS_FP64_IEEE) {
        AcuIeee<double>::C c{dt / rho, dt * k, {make_div(dx), make_div(dy), make_div(dz)}};
        return launch_acoustic<AcuIeee<double>>(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, c, st, s);
    }
    if (fp64_mode != PS_FP64_SPLIT)
        return fail(PS_ERR_UNSUPPORTED, "ps_acoustic3d_step: fp64_mode %d (IEEE or SPLIT)", fp64_mode);
    const double h[3] = {dx, dy, dz};
    AcuSplit::C c;
    // (dt/ρ)/h and (dt·k)/h to ~106 bits, from the FP64 values dt/ρ and dt·k the reference's
    // statements form first (their one rounding is then the same in both arithmetics)
    const double dtr = dt / rho, dtk = dt * k;
    for (int d = 0; d < 3; ++d) {
        double hi, lo;
        div2_host(dtr, h[d], &hi, &lo);
        split3_host(hi, lo, &c.cv[d], &c.cvr[d]);
        div2_host(dtk, h[d], &hi, &lo);
        split3_host(hi, lo, &c.ck[d], &c.ckr[d]);
    }
    return launch_acoustic<AcuSplit>(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, c, st, s);
}

// The second state set of ps_acoustic3d_run: grow-only, one per device and stream.
struct AcuScratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};
std::mutex g_acu_mutex;
std::map<std::pair<int, cudaStream_t>, AcuScratch> g_acu_scratch;

int acu_scratch(size_t bytes, void** p, cudaStream_t s) {
    int dev = 0;
    PS_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_acu_mutex);
    AcuScratch& sc = g_acu_scratch[{dev, s}];
    if (sc.bytes < bytes) {
        if (sc.ptr) {
            PS_CUDA_TRY(cudaStreamSynchronize(s));
            PS_CUDA_TRY(cudaFree(sc.ptr));
            sc.ptr = nullptr;
            sc.bytes = 0;
        }
        PS_CUDA_TRY(cudaMalloc(&sc.ptr, bytes));
        sc.bytes = bytes;
    }
    *p = sc.ptr;
    return PS_OK;
}

}  // namespace

void acoustic_free_scratch() {
    std::lock_guard<std::mutex> lk(g_acu_mutex);
    for (auto& kv : g_acu_scratch)
        if (kv.second.ptr) cudaFree(kv.second.ptr);
    g_acu_scratch.clear();
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_acoustic3d_step(ps_array Vx, ps_array Vy, ps_array Vz, ps_array P, ps_array Vx2, ps_array Vy2, ps_array Vz2,
                       ps_array P2, double dt, double rho, double k, double dx, double dy, double dz,
                       int32_t fp64_mode, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_acoustic(Vx, Vy, Vz, P, kNames));
    PS_TRY(check_acoustic(Vx2, Vy2, Vz2, P2, kNames2));
    PS_TRY(check_same_dtype(P, P2, "P", "P2"));
    PS_TRY(check_shape(P2, P.n[0], P.n[1], P.n[2], "P2"));
    const ps_array in[4] = {Vx, Vy, Vz, P}, out[4] = {Vx2, Vy2, Vz2, P2};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            if (overlaps(in[i], out[j]) || (i < j && (overlaps(out[i], out[j]))))
                return fail(PS_ERR_ARG, "ps_acoustic3d_step: the output arrays overlap each other or the inputs");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_TRY(acoustic_step(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, dt, rho, k, dx, dy, dz, fp64_mode, st, s));
    return finish_launch(s, sync, "ps_acoustic3d_step");
}

int ps_acoustic3d_run(ps_array Vx, ps_array Vy, ps_array Vz, ps_array P, double dt, double rho, double k, double dx,
                      double dy, double dz, int64_t nt, int32_t fp64_mode, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_acoustic(Vx, Vy, Vz, P, kNames));
    if (nt < 0) return fail(PS_ERR_ARG, "ps_acoustic3d_run: nt = %lld < 0", (long long)nt);
    if (nt == 0) return PS_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t es = elsize(P.dtype);
    const size_t b[4] = {(size_t)numel(Vx) * es, (size_t)numel(Vy) * es, (size_t)numel(Vz) * es,
                         (size_t)numel(P) * es};
    size_t off[4], total = 0;
    for (int i = 0; i < 4; ++i) {
        off[i] = total;
        total += (b[i] + 255) / 256 * 256;
    }
    if (P.dtype == PS_F64 && fp64_mode == PS_FP64_IEEE) {
        // IEEE FP64 is bound by the FP64 pipe, where the fused kernel's extra face updates (the Vy
        // face of the next row, the Vx face past each warp) cost more than its saved traffic: the
        // miniapp's two kernels in place (measured 1.73 against 2.50 ms per step at 255^3)
        for (int64_t it = 0; it < nt; ++it) {
            PS_TRY(ps_acoustic3d_v(Vx, Vy, Vz, P, dt, rho, dx, dy, dz, stream, 0));
            PS_TRY(ps_acoustic3d_p(P, Vx, Vy, Vz, dt, k, dx, dy, dz, stream, 0));
        }
        return PS_OK;
    }
    void* base = nullptr;
    PS_TRY(acu_scratch(total, &base, s));
    ps_array B[4] = {Vx, Vy, Vz, P};
    for (int i = 0; i < 4; ++i) B[i].ptr = static_cast<char*>(base) + off[i];
    const ps_array A[4] = {Vx, Vy, Vz, P};
    for (int64_t it = 0; it < nt; ++it) {
        const ps_array* src = (it % 2 == 0) ? A : B;
        const ps_array* dst = (it % 2 == 0) ? B : A;
        PS_TRY(acoustic_step(src[0], src[1], src[2], src[3], dst[0], dst[1], dst[2], dst[3], dt, rho, k, dx, dy, dz,
                             fp64_mode, st, s));
        PS_TRY(finish_launch(s, 0, "ps_acoustic3d_run"));
    }
    if (nt % 2 == 1)  // the last step wrote the library's set
        for (int i = 0; i < 4; ++i) PS_CUDA_TRY(cudaMemcpyAsync(A[i].ptr, B[i].ptr, b[i], cudaMemcpyDeviceToDevice, s));
    return finish_launch(s, 0, "ps_acoustic3d_run");
}

}  // extern "C"
