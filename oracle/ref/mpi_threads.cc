// mpi_threads.cc - thread-rank MPI shim (see mpi.h). TEST INFRASTRUCTURE.
#include "mpi.h"

#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

enum Kind { K_CHAR, K_UCHAR, K_SHORT, K_USHORT, K_INT, K_UNSIGNED, K_LONG, K_ULONG, K_FLOAT,
            K_DOUBLE, K_LDOUBLE, K_LLONG, K_BYTE };

struct shim_type {
  size_t size;
  int kind;
};

shim_type shim_type_char = {sizeof(char), K_CHAR};
shim_type shim_type_uchar = {sizeof(unsigned char), K_UCHAR};
shim_type shim_type_short = {sizeof(short), K_SHORT};
shim_type shim_type_ushort = {sizeof(unsigned short), K_USHORT};
shim_type shim_type_int = {sizeof(int), K_INT};
shim_type shim_type_unsigned = {sizeof(unsigned), K_UNSIGNED};
shim_type shim_type_long = {sizeof(long), K_LONG};
shim_type shim_type_ulong = {sizeof(unsigned long), K_ULONG};
shim_type shim_type_float = {sizeof(float), K_FLOAT};
shim_type shim_type_double = {sizeof(double), K_DOUBLE};
shim_type shim_type_long_double = {sizeof(long double), K_LDOUBLE};
shim_type shim_type_long_long = {sizeof(long long), K_LLONG};
shim_type shim_type_byte = {1, K_BYTE};

struct shim_group {
  std::vector<int> world;  // world ranks, in group order
};

struct shim_comm {
  std::vector<int> members;  // comm rank -> world rank
  int id = 0;
  std::mutex mu;
  std::condition_variable cv;
  int arrived = 0;
  unsigned long long generation = 0;
  // collective scratch, one slot per comm rank
  std::vector<const void*> p0, p1, p2;
  std::vector<long long> v0, v1;
  std::vector<shim_comm*> made;
  explicit shim_comm(const std::vector<int>& m) : members(m) {
    const size_t n = m.size();
    p0.resize(n); p1.resize(n); p2.resize(n); v0.resize(n); v1.resize(n); made.resize(n);
  }
};

struct shim_request {
  bool is_recv = false;
  bool done = false;
  void* buf = nullptr;
  size_t bytes = 0;
  int src = 0;
  int tag = 0;
  shim_comm* comm = nullptr;
  MPI_Status st{};
};

namespace {

struct Msg {
  int comm_id;
  int src;  // comm rank of the sender
  int tag;
  std::vector<char> data;
};

struct Mailbox {
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Msg> q;
};

thread_local int tl_world_rank = 0;
shim_comm* g_world = nullptr;
std::vector<std::unique_ptr<Mailbox>> g_boxes;
std::mutex g_id_mu;
int g_next_id = 1;

int next_id() {
  std::lock_guard<std::mutex> l(g_id_mu);
  return g_next_id++;
}

int my_rank(shim_comm* c) {
  for (size_t i = 0; i < c->members.size(); ++i)
    if (c->members[i] == tl_world_rank) return int(i);
  return -1;
}

void barrier(shim_comm* c) {
  std::unique_lock<std::mutex> l(c->mu);
  const unsigned long long gen = c->generation;
  if (++c->arrived == int(c->members.size())) {
    c->arrived = 0;
    c->generation++;
    c->cv.notify_all();
  } else {
    c->cv.wait(l, [&] { return c->generation != gen; });
  }
}

template <typename T>
void reduce_into(T* acc, const T* x, int n, MPI_Op op) {
  for (int i = 0; i < n; ++i) {
    if (op == MPI_SUM) acc[i] = acc[i] + x[i];
    else if (op == MPI_MAX) acc[i] = std::max(acc[i], x[i]);
    else if (op == MPI_MIN) acc[i] = std::min(acc[i], x[i]);
  }
}

void reduce(void* acc, const void* x, int n, MPI_Datatype t, MPI_Op op) {
  switch (t->kind) {
    case K_CHAR: reduce_into((char*)acc, (const char*)x, n, op); break;
    case K_UCHAR: reduce_into((unsigned char*)acc, (const unsigned char*)x, n, op); break;
    case K_SHORT: reduce_into((short*)acc, (const short*)x, n, op); break;
    case K_USHORT: reduce_into((unsigned short*)acc, (const unsigned short*)x, n, op); break;
    case K_INT: reduce_into((int*)acc, (const int*)x, n, op); break;
    case K_UNSIGNED: reduce_into((unsigned*)acc, (const unsigned*)x, n, op); break;
    case K_LONG: reduce_into((long*)acc, (const long*)x, n, op); break;
    case K_ULONG: reduce_into((unsigned long*)acc, (const unsigned long*)x, n, op); break;
    case K_FLOAT: reduce_into((float*)acc, (const float*)x, n, op); break;
    case K_DOUBLE: reduce_into((double*)acc, (const double*)x, n, op); break;
    case K_LDOUBLE: reduce_into((long double*)acc, (const long double*)x, n, op); break;
    case K_LLONG: reduce_into((long long*)acc, (const long long*)x, n, op); break;
    default: std::fprintf(stderr, "mpi shim: reduction on a byte type\n"); std::abort();
  }
}

void post(shim_comm* c, int dest, int tag, const void* buf, size_t bytes) {
  Msg m;
  m.comm_id = c->id;
  m.src = my_rank(c);
  m.tag = tag;
  m.data.assign((const char*)buf, (const char*)buf + bytes);
  Mailbox& b = *g_boxes[c->members[dest]];
  {
    std::lock_guard<std::mutex> l(b.mu);
    b.q.push_back(std::move(m));
  }
  b.cv.notify_all();
}

// Take the first message matching (comm, src, tag); block when `wait`.
bool take(shim_comm* c, int src, int tag, void* buf, size_t cap, MPI_Status* st, bool wait) {
  Mailbox& b = *g_boxes[tl_world_rank];
  std::unique_lock<std::mutex> l(b.mu);
  while (true) {
    for (auto it = b.q.begin(); it != b.q.end(); ++it) {
      if (it->comm_id != c->id) continue;
      if (src != MPI_ANY_SOURCE && it->src != src) continue;
      if (tag != MPI_ANY_TAG && it->tag != tag) continue;
      const size_t nb = std::min(cap, it->data.size());
      if (nb) std::memcpy(buf, it->data.data(), nb);
      if (st) {
        st->MPI_SOURCE = it->src;
        st->MPI_TAG = it->tag;
        st->MPI_ERROR = MPI_SUCCESS;
        st->count_bytes = (long long)it->data.size();
      }
      b.q.erase(it);
      return true;
    }
    if (!wait) return false;
    b.cv.wait(l);
  }
}

}  // namespace

extern "C" {

MPI_Comm shim_comm_world(void) { return g_world; }

void shim_run_ranks(int nranks, void (*fn)(void*, int), void* arg) {
  std::vector<int> m(nranks);
  for (int i = 0; i < nranks; ++i) m[i] = i;
  g_world = new shim_comm(m);
  g_world->id = next_id();
  g_boxes.clear();
  for (int i = 0; i < nranks; ++i) g_boxes.emplace_back(new Mailbox());
  std::vector<std::thread> ts;
  for (int r = 0; r < nranks; ++r) {
    ts.emplace_back([=] {
      tl_world_rank = r;
      fn(arg, r);
    });
  }
  for (auto& t : ts) t.join();
}

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }

int MPI_Abort(MPI_Comm, int code) {
  std::fprintf(stderr, "MPI_Abort(%d) in the thread-rank shim\n", code);
  std::abort();
}

int MPI_Comm_rank(MPI_Comm c, int* r) {
  *r = my_rank(c);
  return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm c, int* s) {
  *s = int(c->members.size());
  return MPI_SUCCESS;
}

int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out) {
  const int r = my_rank(c), n = int(c->members.size());
  c->v0[r] = color;
  c->v1[r] = key;
  barrier(c);
  int leader = -1;
  std::vector<std::pair<long long, int>> mine;
  for (int i = 0; i < n; ++i) {
    if (c->v0[i] == color) {
      if (leader < 0) leader = i;
      mine.push_back({c->v1[i], i});
    }
  }
  if (leader == r) {
    std::stable_sort(mine.begin(), mine.end());
    std::vector<int> m;
    for (auto& p : mine) m.push_back(c->members[p.second]);
    shim_comm* nc = new shim_comm(m);
    nc->id = next_id();
    c->made[r] = nc;
  }
  barrier(c);
  *out = c->made[leader];
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Comm_group(MPI_Comm c, MPI_Group* g) {
  shim_group* x = new shim_group();
  x->world = c->members;
  *g = x;
  return MPI_SUCCESS;
}

int MPI_Group_incl(MPI_Group g, int n, const int* ranks, MPI_Group* out) {
  shim_group* x = new shim_group();
  for (int i = 0; i < n; ++i) x->world.push_back(g->world[ranks[i]]);
  *out = x;
  return MPI_SUCCESS;
}

int MPI_Comm_create(MPI_Comm c, MPI_Group g, MPI_Comm* out) {
  const int r = my_rank(c), n = int(c->members.size());
  c->p0[r] = g;
  barrier(c);
  const bool member = std::find(g->world.begin(), g->world.end(), tl_world_rank) != g->world.end();
  if (member && !g->world.empty() && g->world[0] == tl_world_rank) {
    shim_comm* nc = new shim_comm(g->world);
    nc->id = next_id();
    c->made[r] = nc;
  }
  barrier(c);
  *out = MPI_COMM_NULL;
  if (member) {
    for (int i = 0; i < n; ++i)
      if (c->members[i] == g->world[0]) *out = c->made[i];
  }
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Comm_free(MPI_Comm* c) {
  *c = MPI_COMM_NULL;  // communicators of the shim live until exit
  return MPI_SUCCESS;
}

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* nt) {
  shim_type* t = new shim_type();
  t->size = size_t(count) * old->size;
  t->kind = K_BYTE;
  *nt = t;
  return MPI_SUCCESS;
}

int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

int MPI_Barrier(MPI_Comm c) {
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm c) {
  const int r = my_rank(c);
  c->p0[r] = buf;
  barrier(c);
  if (r != root) std::memcpy(buf, c->p0[root], size_t(count) * t->size);
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Gather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt,
               int root, MPI_Comm c) {
  const int r = my_rank(c), n = int(c->members.size());
  c->p0[r] = sb;
  barrier(c);
  if (r == root)
    for (int i = 0; i < n; ++i)
      std::memcpy((char*)rb + size_t(i) * rc * rt->size, c->p0[i], size_t(sc) * st->size);
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Allgather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt,
                  MPI_Comm c) {
  const int r = my_rank(c), n = int(c->members.size());
  c->p0[r] = sb;
  barrier(c);
  for (int i = 0; i < n; ++i)
    std::memcpy((char*)rb + size_t(i) * rc * rt->size, c->p0[i], size_t(sc) * st->size);
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Allgatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int* rcs,
                   const int* displs, MPI_Datatype rt, MPI_Comm c) {
  const int r = my_rank(c), n = int(c->members.size());
  c->p0[r] = sb;
  c->v0[r] = sc;
  barrier(c);
  for (int i = 0; i < n; ++i) {
    const size_t cnt = size_t(std::min<long long>(c->v0[i], rcs[i]));
    if (cnt) std::memcpy((char*)rb + size_t(displs[i]) * rt->size, c->p0[i], cnt * st->size);
  }
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Allreduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  const int r = my_rank(c), n = int(c->members.size());
  c->p0[r] = sb;
  barrier(c);
  std::vector<char> acc((const char*)c->p0[0], (const char*)c->p0[0] + size_t(count) * t->size);
  for (int i = 1; i < n; ++i) reduce(acc.data(), c->p0[i], count, t, op);
  barrier(c);
  std::memcpy(rb, acc.data(), acc.size());
  return MPI_SUCCESS;
}

int MPI_Scan(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  const int r = my_rank(c);
  c->p0[r] = sb;
  barrier(c);
  std::vector<char> acc((const char*)c->p0[0], (const char*)c->p0[0] + size_t(count) * t->size);
  for (int i = 1; i <= r; ++i) reduce(acc.data(), c->p0[i], count, t, op);
  barrier(c);
  std::memcpy(rb, acc.data(), acc.size());
  return MPI_SUCCESS;
}

int MPI_Alltoall(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt,
                 MPI_Comm c) {
  const int r = my_rank(c), n = int(c->members.size());
  c->p0[r] = sb;
  barrier(c);
  for (int i = 0; i < n; ++i)
    std::memcpy((char*)rb + size_t(i) * rc * rt->size,
                (const char*)c->p0[i] + size_t(r) * sc * st->size, size_t(sc) * st->size);
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Alltoallv(const void* sb, const int* scs, const int* sds, MPI_Datatype st, void* rb,
                  const int* rcs, const int* rds, MPI_Datatype rt, MPI_Comm c) {
  const int r = my_rank(c), n = int(c->members.size());
  c->p0[r] = sb;
  c->p1[r] = scs;
  c->p2[r] = sds;
  barrier(c);
  for (int i = 0; i < n; ++i) {
    const int cnt = ((const int*)c->p1[i])[r];
    const int off = ((const int*)c->p2[i])[r];
    const size_t nb = size_t(std::min(cnt, rcs[i])) * st->size;
    if (nb) std::memcpy((char*)rb + size_t(rds[i]) * rt->size,
                        (const char*)c->p0[i] + size_t(off) * st->size, nb);
  }
  barrier(c);
  return MPI_SUCCESS;
}

int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c) {
  post(c, dest, tag, buf, size_t(count) * t->size);
  return MPI_SUCCESS;
}

int MPI_Recv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c,
             MPI_Status* st) {
  take(c, src, tag, buf, size_t(count) * t->size, st, true);
  return MPI_SUCCESS;
}

int MPI_Sendrecv(const void* sb, int sc, MPI_Datatype stp, int dest, int stag, void* rb, int rc,
                 MPI_Datatype rtp, int src, int rtag, MPI_Comm c, MPI_Status* st) {
  post(c, dest, stag, sb, size_t(sc) * stp->size);
  take(c, src, rtag, rb, size_t(rc) * rtp->size, st, true);
  return MPI_SUCCESS;
}

int MPI_Issend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c,
               MPI_Request* req) {
  post(c, dest, tag, buf, size_t(count) * t->size);
  shim_request* q = new shim_request();
  q->done = true;
  *req = q;
  return MPI_SUCCESS;
}

int MPI_Irecv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c,
              MPI_Request* req) {
  shim_request* q = new shim_request();
  q->is_recv = true;
  q->buf = buf;
  q->bytes = size_t(count) * t->size;
  q->src = src;
  q->tag = tag;
  q->comm = c;
  *req = q;
  return MPI_SUCCESS;
}

int MPI_Test(MPI_Request* req, int* flag, MPI_Status* st) {
  shim_request* q = *req;
  if (!q) { *flag = 1; return MPI_SUCCESS; }
  if (!q->done && q->is_recv) q->done = take(q->comm, q->src, q->tag, q->buf, q->bytes, &q->st, false);
  *flag = q->done ? 1 : 0;
  if (q->done && st) *st = q->st;
  return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request* req, MPI_Status* st) {
  shim_request* q = *req;
  if (!q) return MPI_SUCCESS;
  if (!q->done && q->is_recv) q->done = take(q->comm, q->src, q->tag, q->buf, q->bytes, &q->st, true);
  if (st) *st = q->st;
  return MPI_SUCCESS;
}

int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* sts) {
  for (int i = 0; i < n; ++i) MPI_Wait(&reqs[i], sts ? &sts[i] : MPI_STATUS_IGNORE);
  return MPI_SUCCESS;
}

}  // extern "C"
