// Run-time side of the stand-ins that let the reference's own sources build
// and run here as a parity pin for the oracle (test infrastructure; nothing
// in the product links it): MPI for one rank, and the FFTW-MPI plans the
// reference creates, computed with a project-written discrete Fourier
// transform.  The headers under include/ state the semantics.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <vector>

#include <fftw3-mpi.h>
#include <mpi.h>

// ------------------------------------------------------------------ MPI
namespace {

size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_CHAR: return 1;
    case MPI_BYTE: return 1;
    case MPI_C_BOOL: return sizeof(bool);
    case MPI_LONG_LONG: return sizeof(long long);
    case MPI_UNSIGNED_LONG: return sizeof(unsigned long);
    case MPI_UNSIGNED: return sizeof(unsigned);
    case MPI_LONG: return sizeof(long);
  }
  std::fprintf(stderr, "refpin MPI: unknown datatype %d\n", t);
  std::abort();
}

void check_rank(int r, const char* what) {
  if (r != 0) {
    std::fprintf(stderr, "refpin MPI: %s addresses rank %d of a one-rank world\n", what, r);
    std::abort();
  }
}

struct Message {
  int tag;
  std::vector<char> bytes;
};
struct PendingRecv {
  void* buf;
  size_t bytes;
  int tag;
  bool done;
};

std::deque<Message> g_queue;            // sent, not yet received
std::map<int, PendingRecv> g_recvs;     // posted receives by request id
int g_next_req = 1;

bool match(PendingRecv& r) {
  for (auto it = g_queue.begin(); it != g_queue.end(); ++it) {
    if (it->tag != r.tag) continue;
    if (it->bytes.size() > r.bytes) {
      std::fprintf(stderr, "refpin MPI: message of %zu bytes into a %zu-byte receive\n", it->bytes.size(), r.bytes);
      std::abort();
    }
    if (!it->bytes.empty()) std::memcpy(r.buf, it->bytes.data(), it->bytes.size());
    g_queue.erase(it);
    r.done = true;
    return true;
  }
  return false;
}

void deliver(const void* buf, size_t bytes, int tag) {
  g_queue.push_back(Message{tag, std::vector<char>((const char*)buf, (const char*)buf + bytes)});
  for (auto& kv : g_recvs)
    if (!kv.second.done && match(kv.second)) break;
}

}  // namespace

extern "C" {

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
int MPI_Bcast(void*, int, MPI_Datatype, int root, MPI_Comm) { check_rank(root, "MPI_Bcast"); return MPI_SUCCESS; }

int MPI_Allreduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (sbuf != rbuf) std::memmove(rbuf, sbuf, (size_t)count * type_size(t));
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  check_rank(root, "MPI_Reduce");
  return MPI_Allreduce(sbuf, rbuf, count, t, op, c);
}
int MPI_Gather(const void* sbuf, int scount, MPI_Datatype st, void* rbuf, int, MPI_Datatype, int root, MPI_Comm) {
  check_rank(root, "MPI_Gather");
  if (sbuf != rbuf) std::memmove(rbuf, sbuf, (size_t)scount * type_size(st));
  return MPI_SUCCESS;
}
int MPI_Gatherv(const void* sbuf, int scount, MPI_Datatype st, void* rbuf, const int*, const int* displs,
                MPI_Datatype rt, int root, MPI_Comm) {
  check_rank(root, "MPI_Gatherv");
  std::memmove((char*)rbuf + (size_t)displs[0] * type_size(rt), sbuf, (size_t)scount * type_size(st));
  return MPI_SUCCESS;
}

int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm) {
  check_rank(dest, "MPI_Send");
  deliver(buf, (size_t)count * type_size(t), tag);
  return MPI_SUCCESS;
}
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c, MPI_Request* req) {
  MPI_Send(buf, count, t, dest, tag, c);  // buffered: complete at once
  *req = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm, MPI_Request* req) {
  check_rank(source, "MPI_Irecv");
  const int id = g_next_req++;
  PendingRecv r{buf, (size_t)count * type_size(t), tag, false};
  match(r);
  g_recvs[id] = r;
  *req = id;
  return MPI_SUCCESS;
}
int MPI_Test(MPI_Request* req, int* flag, MPI_Status*) {
  if (*req == MPI_REQUEST_NULL) { *flag = 1; return MPI_SUCCESS; }
  auto it = g_recvs.find(*req);
  if (it == g_recvs.end()) { *flag = 1; *req = MPI_REQUEST_NULL; return MPI_SUCCESS; }
  if (!it->second.done) match(it->second);
  *flag = it->second.done ? 1 : 0;
  if (*flag) { g_recvs.erase(it); *req = MPI_REQUEST_NULL; }
  return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request* req, MPI_Status* st) {
  int flag = 0;
  MPI_Test(req, &flag, st);
  if (!flag) {
    std::fprintf(stderr, "refpin MPI: a receive waits for a message that was never sent\n");
    std::abort();
  }
  return MPI_SUCCESS;
}
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status*) {
  for (int i = 0; i < n; ++i) MPI_Wait(reqs + i, MPI_STATUS_IGNORE);
  return MPI_SUCCESS;
}
int MPI_Recv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm c, MPI_Status* st) {
  MPI_Request r;
  MPI_Irecv(buf, count, t, source, tag, c, &r);
  return MPI_Wait(&r, st);
}
int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype st, int dest, int stag, void* rbuf, int rcount,
                 MPI_Datatype rt, int source, int rtag, MPI_Comm c, MPI_Status* status) {
  MPI_Send(sbuf, scount, st, dest, stag, c);
  return MPI_Recv(rbuf, rcount, rt, source, rtag, c, status);
}

}  // extern "C"

// ------------------------------------------------------------------ FFTW
// Unnormalised DFT of one line: X[k] = sum_n x[n] exp(sign 2 pi i k n / N),
// by a radix-2 Cooley-Tukey recursion for even lengths and the direct sum
// otherwise; twiddles from long-double sine and cosine.
namespace {

using cd = std::complex<double>;

void dft(std::vector<cd>& a, int sign) {
  const size_t n = a.size();
  if (n <= 1) return;
  if (n % 2 == 0) {
    std::vector<cd> e(n / 2), o(n / 2);
    for (size_t i = 0; i < n / 2; ++i) {
      e[i] = a[2 * i];
      o[i] = a[2 * i + 1];
    }
    dft(e, sign);
    dft(o, sign);
    for (size_t k = 0; k < n / 2; ++k) {
      const long double ang = (long double)sign * 2.0L * 3.141592653589793238462643383279502884L * k / n;
      const cd w((double)std::cos(ang), (double)std::sin(ang));
      const cd t = w * o[k];
      a[k] = e[k] + t;
      a[k + n / 2] = e[k] - t;
    }
    return;
  }
  std::vector<cd> out(n);
  for (size_t k = 0; k < n; ++k) {
    cd s(0.0, 0.0);
    for (size_t m = 0; m < n; ++m) {
      const long double ang = (long double)sign * 2.0L * 3.141592653589793238462643383279502884L * ((k * m) % n) / n;
      s += a[m] * cd((double)std::cos(ang), (double)std::sin(ang));
    }
    out[k] = s;
  }
  a = out;
}

}  // namespace

struct refpin_plan {
  bool r2c;
  ptrdiff_t n0, n1, n2;
  double* real;      // [n0][n1][2 (n2/2 + 1)]
  fftw_complex* cx;  // [n1][n0][n2/2 + 1]
};

extern "C" {

void fftw_mpi_init(void) {}
void fftw_mpi_cleanup(void) {}
void* fftw_malloc(size_t n) { return std::malloc(n); }
void fftw_free(void* p) { std::free(p); }

ptrdiff_t fftw_mpi_local_size_3d_transposed(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm, ptrdiff_t* local_n0,
                                            ptrdiff_t* local_0_start, ptrdiff_t* local_n1,
                                            ptrdiff_t* local_1_start) {
  *local_n0 = n0;
  *local_0_start = 0;
  *local_n1 = n1;
  *local_1_start = 0;
  return n0 * n1 * (n2 / 2 + 1);
}

fftw_plan fftw_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double* in, fftw_complex* out, MPI_Comm,
                                   unsigned flags) {
  if (!(flags & FFTW_MPI_TRANSPOSED_OUT)) {
    std::fprintf(stderr, "refpin FFTW: only transposed-output r2c plans are provided\n");
    std::abort();
  }
  return new refpin_plan{true, n0, n1, n2, in, out};
}

fftw_plan fftw_mpi_plan_dft_c2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, fftw_complex* in, double* out, MPI_Comm,
                                   unsigned flags) {
  if (!(flags & FFTW_MPI_TRANSPOSED_IN)) {
    std::fprintf(stderr, "refpin FFTW: only transposed-input c2r plans are provided\n");
    std::abort();
  }
  return new refpin_plan{false, n0, n1, n2, out, in};
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

void fftw_execute(const fftw_plan p) {
  const ptrdiff_t n0 = p->n0, n1 = p->n1, n2 = p->n2, h = n2 / 2 + 1, row = 2 * h;
  auto R = [&](ptrdiff_t i0, ptrdiff_t i1, ptrdiff_t i2) -> double& { return p->real[(i0 * n1 + i1) * row + i2]; };
  auto C = [&](ptrdiff_t k1, ptrdiff_t k0, ptrdiff_t k2) -> cd& {
    return reinterpret_cast<cd*>(p->cx)[(k1 * n0 + k0) * h + k2];
  };
  // work array W[k2][i0][i1] of the half spectrum along the last axis
  std::vector<cd> W((size_t)(h * n0 * n1));
  auto w = [&](ptrdiff_t k2, ptrdiff_t i0, ptrdiff_t i1) -> cd& { return W[(size_t)((k2 * n0 + i0) * n1 + i1)]; };
  if (p->r2c) {
    std::vector<cd> line((size_t)n2);
    for (ptrdiff_t i0 = 0; i0 < n0; ++i0)
      for (ptrdiff_t i1 = 0; i1 < n1; ++i1) {
        for (ptrdiff_t i2 = 0; i2 < n2; ++i2) line[(size_t)i2] = cd(R(i0, i1, i2), 0.0);
        dft(line, -1);
        for (ptrdiff_t k2 = 0; k2 < h; ++k2) w(k2, i0, i1) = line[(size_t)k2];
      }
    std::vector<cd> l1((size_t)n1), l0((size_t)n0);
    for (ptrdiff_t k2 = 0; k2 < h; ++k2) {
      for (ptrdiff_t i0 = 0; i0 < n0; ++i0) {
        for (ptrdiff_t i1 = 0; i1 < n1; ++i1) l1[(size_t)i1] = w(k2, i0, i1);
        dft(l1, -1);
        for (ptrdiff_t i1 = 0; i1 < n1; ++i1) w(k2, i0, i1) = l1[(size_t)i1];
      }
      for (ptrdiff_t k1 = 0; k1 < n1; ++k1) {
        for (ptrdiff_t i0 = 0; i0 < n0; ++i0) l0[(size_t)i0] = w(k2, i0, k1);
        dft(l0, -1);
        for (ptrdiff_t k0 = 0; k0 < n0; ++k0) C(k1, k0, k2) = l0[(size_t)k0];
      }
    }
  } else {
    std::vector<cd> l1((size_t)n1), l0((size_t)n0);
    for (ptrdiff_t k2 = 0; k2 < h; ++k2) {
      for (ptrdiff_t k1 = 0; k1 < n1; ++k1) {
        for (ptrdiff_t k0 = 0; k0 < n0; ++k0) l0[(size_t)k0] = C(k1, k0, k2);
        dft(l0, +1);
        for (ptrdiff_t i0 = 0; i0 < n0; ++i0) w(k2, i0, k1) = l0[(size_t)i0];
      }
      for (ptrdiff_t i0 = 0; i0 < n0; ++i0) {
        for (ptrdiff_t k1 = 0; k1 < n1; ++k1) l1[(size_t)k1] = w(k2, i0, k1);
        dft(l1, +1);
        for (ptrdiff_t i1 = 0; i1 < n1; ++i1) w(k2, i0, i1) = l1[(size_t)i1];
      }
    }
    // real inverse along the last axis from the half spectrum: the entries
    // kx = 0 and kx = n2/2 contribute their real parts only
    std::vector<cd> line((size_t)n2);
    for (ptrdiff_t i0 = 0; i0 < n0; ++i0)
      for (ptrdiff_t i1 = 0; i1 < n1; ++i1) {
        for (ptrdiff_t k2 = 0; k2 < n2; ++k2) {
          if (k2 < h) {
            cd v = w(k2, i0, i1);
            if (k2 == 0 || 2 * k2 == n2) v = cd(v.real(), 0.0);
            line[(size_t)k2] = v;
          } else {
            line[(size_t)k2] = std::conj(w(n2 - k2, i0, i1));
          }
        }
        dft(line, +1);
        for (ptrdiff_t i2 = 0; i2 < n2; ++i2) R(i0, i1, i2) = line[(size_t)i2].real();
      }
  }
}

}  // extern "C"
