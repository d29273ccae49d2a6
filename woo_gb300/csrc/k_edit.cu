// k_edit.cu -- particle removal and insertion on the device, between steps: the GB300 counterpart of
// DemField::removeParticle (src/dem/Particle.cpp:483-530, called by Outlet::run, src/dem/Outlet.cpp:15-116)
// and of particles added by RandomInlet::run (src/dem/Inlet.cpp:228-515).  Only the changed slots and the
// contacts of removed particles are touched; the rest of the particle and contact state stays on the device.
//
// A removed particle's slot stays allocated (Woo keeps the id free for ParticleContainer::findFreeId): it
// becomes inert, with mask 0 so that Collider::mayCollide (src/dem/Collision.cpp:21-43) never pairs it, all
// DOFs blocked and no velocity, optionally parked at a given position (so that a particle removed far from
// the others does not stretch the collider's grid).  Its contacts die with their history, as
// ContactContainer::remove drops them.
#include "wdem_internal.h"
#include "wdem_math.cuh"
#include "../../include/wdem.h"

namespace wdem {

__global__ void k_kill_slots(Particles p, const int* ids, int m, const double* park, uint8_t* gone) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int i = ids[k];
  gone[i] = 1;
  int4 meta = p.meta[i];
  meta.z = 0;
  meta.w |= 63;
  p.meta[i] = meta;
  double4_32a v = p.velm[i];
  v.x = 0; v.y = 0; v.z = 0;
  p.velm[i] = v;
  double4_32a w = p.angw[i];
  w.x = 0; w.y = 0; w.z = 0;
  p.angw[i] = w;
  if (park) {
    double4_32a pr = p.posr[i];
    pr.x = park[3 * k]; pr.y = park[3 * k + 1]; pr.z = park[3 * k + 2];
    p.posr[i] = pr;
    p.posf[i] = make_float4((float)pr.x, (float)pr.y, (float)pr.z, (float)pr.w);
  }
  p.force[i] = make_double4_32a(0, 0, 0, 0);
  p.torque[i] = make_double4_32a(0, 0, 0, 0);
  p.touched[i] = 0;
  p.rowMask[i] = 0;
}

__global__ void k_kill_contacts(Contacts c, long long nc, const uint8_t* gone) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const int2 id = c.ids[i];
  if (gone[id.x] || gone[id.y]) {
    const uint8_t s = c.state[i];
    if ((s & CS_MASK) != CS_DEAD) c.state[i] = (uint8_t)(CS_DEAD | (s & CS_SHAPES));
  }
}

__global__ void k_clear_gone(const int* ids, int m, uint8_t* gone) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) gone[ids[k]] = 0;
}

// Inserted particles: EDIT_RECORDS records per particle packed on the host (posr, velm, angw, inert, ori,
// force, torque; then semi-axes and angMom when the handle tracks rotation state), scattered to their slots.
__global__ void k_put_slots(Particles p, const int* ids, int m, const double4_32a* rec, const int4* meta, int withRot) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int i = ids[k];
  const double4_32a* r = rec + (long long)EDIT_RECORDS * k;
  p.posr[i] = r[0];
  p.velm[i] = r[1];
  p.angw[i] = r[2];
  p.inert[i] = r[3];
  p.ori[i] = r[4];
  p.force[i] = r[5];
  p.torque[i] = r[6];
  p.meta[i] = meta[k];
  p.lastPos[i] = make_double4_32a(r[0].x, r[0].y, r[0].z, 0);
  p.posf[i] = make_float4((float)r[0].x, (float)r[0].y, (float)r[0].z, (float)r[0].w);
  p.touched[i] = 0;
  p.rowMask[i] = 0;
  if (withRot) {
    p.semi[i] = r[7];
    p.angMom[i] = r[8];
  }
}

void launch_kill(cudaStream_t s, Particles p, int n, const int* ids, int m, const double* park, uint8_t* gone,
                 Contacts c, long long nc) {
  if (m <= 0) return;
  (k_kill_slots<<<(m + 255) / 256, 256, 0, s>>>(p, ids, m, park, gone), ++::wdem::g_kernel_launches);
  if (nc > 0) (k_kill_contacts<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(c, nc, gone), ++::wdem::g_kernel_launches);
  (k_clear_gone<<<(m + 255) / 256, 256, 0, s>>>(ids, m, gone), ++::wdem::g_kernel_launches);
  (void)n;
}

void launch_put(cudaStream_t s, Particles p, const int* ids, int m, const double4_32a* rec, const int4* meta, bool withRot) {
  if (m <= 0) return;
  (k_put_slots<<<(m + 255) / 256, 256, 0, s>>>(p, ids, m, rec, meta, withRot ? 1 : 0), ++::wdem::g_kernel_launches);
}

}  // namespace wdem
