// refhost_driver.cpp - runs the reference's own device functions on the host.
// TEST INFRASTRUCTURE: built only where the reference sources are present
// (never on the GPU host), into oracle/_ref/librefhost.so, and used only by
// tests and the golden-vector script to cross-check the oracle.
//
// The reference's src/sim.cuh is compiled unchanged as C++ (ref_shim/ supplies
// host stand-ins for the CUDA headers and ref_fixes.h the two compile fixes).
// This driver replaces the kernel's thread/cluster machinery
// (mercurius_solver, sim.cuh:615-766): it emulates each thread with a
// thread_local threadIdx, gives every function the block-local arrays the
// kernel passes (SMEM of the thread's block) and a MappedBlock over block 0,
// and runs the phases between the kernel's cluster.sync() calls as
// "every body reads, then every body writes".
#include <vector>

#include "sim.cuh"

thread_local merc_dim3 threadIdx = {0, 0, 0};
thread_local merc_dim3 blockDim = {1, 1, 1};
double merc_ref_hill_factor = 1.0;

namespace {
struct ElemRegs {
  double inc, node, peri, M, e, a;  // the kernel's per-thread element registers
};
}  // namespace

extern "C" {

// One system: n bodies (massive first, nm of them), block size B (the
// reference uses N/16; B = n emulates a single block), elements in
// (6 x n, order inc, node, peri, M, e, a), masses.  Runs the kernel prologue,
// n_steps steps of the loop, and writes heliocentric positions and DH
// velocities (pos/vel 3 x n component-major) and the element registers'
// semi-major axis (a_lag).  If out_elements != NULL it also runs the kernel
// epilogue (reverse DH, elements) and writes the elements.
int refhost_run(int n, int nm, int B, const double* elements, const double* mass, double dt, double hill_factor,
                long n_steps, double* pos, double* vel, double* a_lag, double* out_elements, unsigned char* ce_last) {
  if (n <= 0 || B <= 0 || nm > B || n % B != 0) return 1;
  merc_ref_hill_factor = hill_factor;
  blockDim.x = B;
  std::vector<double3> x(n), v(n), xn(n), vn(n);
  std::vector<double> m(mass, mass + n);
  std::vector<ElemRegs> reg(n);
  std::vector<unsigned char> ce(n, 0);
  MappedBlock mb;
  mb.positions = x.data();  // block 0 holds bodies 0..B-1, the massive ones among them
  mb.velocities = v.data();
  mb.masses = m.data();
  auto set_thread = [&](int j) { threadIdx.x = (unsigned)(j % B); };
  auto base = [&](std::vector<double3>& arr, int j) { return arr.data() + (j / B) * B; };

  // prologue, sim.cuh:654-677
  for (int j = 0; j < n; j++) {
    ElemRegs& b = reg[j];
    b.inc = elements[0 * n + j];
    b.node = elements[1 * n + j];
    b.peri = elements[2 * n + j];
    b.M = elements[3 * n + j];
    b.e = elements[4 * n + j];
    b.a = elements[5 * n + j];
    PosVel pv = cartesian_from_elements(b.inc, b.node, b.peri, b.M, b.e, b.a);
    x[j] = pv.pos;
    v[j] = pv.vel;
  }
  for (int j = 0; j < n; j++) {
    set_thread(j);
    vn[j] = democratic_heliocentric_conversion(PosVel{x[j], v[j]}, nm, &mb);
  }
  v.swap(vn);
  mb.velocities = v.data();

  const double half_dt = 0.5 * dt;
  for (long step = 0; step < n_steps; step++) {
    for (int j = 0; j < n; j++) {
      set_thread(j);
      vn[j] = body_interaction_kick(PosVel{x[j], v[j]}, nm, half_dt, &mb);
    }
    v.swap(vn);
    mb.velocities = v.data();
    for (int j = 0; j < n; j++) {
      set_thread(j);
      xn[j] = main_body_kinetic(base(x, j), nm, half_dt, &mb);
    }
    x.swap(xn);
    mb.positions = x.data();
    for (int j = 0; j < n; j++) {
      set_thread(j);
      ElemRegs& b = reg[j];
      double nmot = rsqrt(b.a * b.a * b.a);
      bool is_ce = close_encounter_p(base(x, j), base(v, j), m.data(), nm, dt, &mb);
      PosVel bs = richardson_extrapolation(PosVel{x[j], v[j]}, nm, dt, &mb);
      elements_from_cartesian(base(x, j), base(v, j), &b.inc, &b.node, &b.peri, &b.M, &b.e, &b.a);
      b.M = (double)(!is_ce) * fmod(fma(nmot, dt, b.M), TWOPI) + (double)(is_ce)*b.M;
      PosVel kep = cartesian_from_elements(b.inc, b.node, b.peri, b.M, b.e, b.a);
      double nce = (1.00 - (double)is_ce);
      xn[j] = make_double3(fma(nce, kep.pos.x, (double)is_ce * bs.pos.x), fma(nce, kep.pos.y, (double)is_ce * bs.pos.y),
                           fma(nce, kep.pos.z, (double)is_ce * bs.pos.z));
      vn[j] = make_double3(fma(nce, kep.vel.x, (double)is_ce * bs.vel.x), fma(nce, kep.vel.y, (double)is_ce * bs.vel.y),
                           fma(nce, kep.vel.z, (double)is_ce * bs.vel.z));
      ce[j] = is_ce;
    }
    x.swap(xn);
    v.swap(vn);
    mb.positions = x.data();
    mb.velocities = v.data();
    for (int j = 0; j < n; j++) {
      set_thread(j);
      xn[j] = main_body_kinetic(base(x, j), nm, half_dt, &mb);
    }
    x.swap(xn);
    mb.positions = x.data();
    for (int j = 0; j < n; j++) {
      set_thread(j);
      vn[j] = body_interaction_kick(PosVel{x[j], v[j]}, nm, half_dt, &mb);
    }
    v.swap(vn);
    mb.velocities = v.data();
  }
  for (int j = 0; j < n; j++) {
    pos[j] = x[j].x; pos[n + j] = x[j].y; pos[2 * n + j] = x[j].z;
    vel[j] = v[j].x; vel[n + j] = v[j].y; vel[2 * n + j] = v[j].z;
    if (a_lag) a_lag[j] = reg[j].a;
    if (ce_last) ce_last[j] = ce[j];
  }
  if (out_elements) {  // epilogue, sim.cuh:746-765
    for (int j = 0; j < n; j++) {
      set_thread(j);
      vn[j] = democratic_heliocentric_conversion(PosVel{x[j], v[j]}, nm, &mb, true);
    }
    v.swap(vn);
    mb.velocities = v.data();
    for (int j = 0; j < n; j++) {
      set_thread(j);
      ElemRegs& b = reg[j];
      elements_from_cartesian(base(x, j), base(v, j), &b.inc, &b.node, &b.peri, &b.M, &b.e, &b.a);
      out_elements[0 * n + j] = b.inc;
      out_elements[1 * n + j] = b.node;
      out_elements[2 * n + j] = b.peri;
      out_elements[3 * n + j] = b.M;
      out_elements[4 * n + j] = b.e;
      out_elements[5 * n + j] = b.a;
    }
  }
  return 0;
}

// Unit-level wrappers of single reference functions.
void refhost_danby(long n, const double* M, const double* e, double* E) {
  for (long i = 0; i < n; i++) E[i] = danby_burkardt(M[i], e[i]);
}

void refhost_cart_from_elem(long n, const double* el, double* pos, double* vel) {
  for (long j = 0; j < n; j++) {
    PosVel pv = cartesian_from_elements(el[j], el[n + j], el[2 * n + j], el[3 * n + j], el[4 * n + j], el[5 * n + j]);
    pos[j] = pv.pos.x; pos[n + j] = pv.pos.y; pos[2 * n + j] = pv.pos.z;
    vel[j] = pv.vel.x; vel[n + j] = pv.vel.y; vel[2 * n + j] = pv.vel.z;
  }
}

void refhost_elem_from_cart(long n, const double* pos, const double* vel, double* el) {
  blockDim.x = 1;
  threadIdx.x = 0;
  for (long j = 0; j < n; j++) {
    double3 p = make_double3(pos[j], pos[n + j], pos[2 * n + j]);
    double3 v = make_double3(vel[j], vel[n + j], vel[2 * n + j]);
    elements_from_cartesian(&p, &v, &el[j], &el[n + j], &el[2 * n + j], &el[3 * n + j], &el[4 * n + j], &el[5 * n + j]);
  }
}

}  // extern "C"
