/*
 * grx_philox.h -- the counter-based random stream of libgrx, for host callers.
 *
 * Every random number the library's kernels use is a Philox4x32-10 draw
 * (Salmon, Moraes, Dror, Shaw, SC'11) with
 *   key     = {seed lo, seed hi}
 *   counter = {slot, move lo, move hi, stream}
 * and uniforms u = word * 2^-32 in [0, 1). gRASPA draws from a pre-filled table
 * (RandomNumber, data_struct.h:1287-1346) and glibc rand(); here a move is a pure
 * function of (seed, stream, move), so a host driver that calls the energy entry
 * points one by one reproduces the device-resident drivers draw for draw.
 *
 * Slots of one move:
 *   GRX_SLOT_FIRST  + t   first-bead trial t: words 0..2 = fractional position
 *   GRX_SLOT_ORIENT + o   trial orientation o: words 0..2 = quaternion uniforms
 *   GRX_SLOT_SELECT       words 0 / 1 = Rosenbluth selection of the first bead /
 *                         of the orientation (words 2 / 3: reinsertion retrace)
 *   GRX_SLOT_RETRACE + o  reinsertion retrace orientation o
 *   GRX_SLOT_MOVE         {molecule pick, move choice, insertion-vs-deletion, acceptance}
 *   GRX_SLOT_DISP         {three displacement / rotation-angle uniforms}
 *   GRX_SLOT_VOLUME       {volume change, acceptance, Gibbs box choice} of a volume move
 *   GRX_SLOT_SWAP         {old component, new component, old molecule, acceptance} of an
 *                         identity swap
 *   GRX_SLOT_GIBBS        {box choice, deletion molecule, acceptance} of a Gibbs particle
 *                         transfer
 */
#ifndef GRX_PHILOX_H
#define GRX_PHILOX_H
#include <stdint.h>

#define GRX_SLOT_FIRST 0u
#define GRX_SLOT_ORIENT 1024u
#define GRX_SLOT_SELECT 2048u
#define GRX_SLOT_RETRACE 3072u
#define GRX_SLOT_MOVE 4096u
#define GRX_SLOT_DISP 4097u
#define GRX_SLOT_VOLUME 4098u
#define GRX_SLOT_SWAP 4099u
#define GRX_SLOT_GIBBS 4100u

static inline void grx_philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

static inline void grx_draw(uint64_t seed, uint32_t stream, uint64_t move, uint32_t slot, uint32_t out[4]) {
  out[0] = slot;
  out[1] = (uint32_t)move;
  out[2] = (uint32_t)(move >> 32);
  out[3] = stream;
  grx_philox4x32_10(out, (uint32_t)seed, (uint32_t)(seed >> 32));
}

static inline double grx_u01(uint32_t w) { return (double)w * 2.3283064365386963e-10; }

#endif /* GRX_PHILOX_H */
