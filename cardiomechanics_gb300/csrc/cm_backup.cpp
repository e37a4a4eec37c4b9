// acCELLerate backup files (acCELLerate::WriteBackup / ReadBackup, acCELLerate.cpp:1511-1661)
// for batches: the two header lines, then per node its Vm and its cell model's GetBase() block.
// The blocks come from cm_batch_get_state / cm_batch_set_state in CM_LAYOUT_REF_BLOCK.
#include <cstdio>
#include <cstring>
#include <strings.h>

#include <string>
#include <vector>

#include "cm_handles.h"

using namespace cm;

namespace {

// acCELLerate.cpp:74
const char kBackupVersion[] = "acCELLerateBackupVersion1.0";

struct Owner {
  int part = -1;
  int64_t local = 0;
};

// Global node -> (part, local index); every node 0 .. n_total-1 exactly once.
int node_owners(int n_parts, const cm_batch_t *parts, const int64_t *const *node_ids, std::vector<Owner> &own) {
  if (n_parts <= 0 || !parts) return fail(CM_ERR_ARG, "need at least one part");
  int64_t total = 0;
  for (int p = 0; p < n_parts; p++) {
    if (!parts[p]) return fail(CM_ERR_ARG, "NULL part " + std::to_string(p));
    total += parts[p]->d.n;
  }
  own.assign((size_t)total, Owner{});
  int64_t next = 0;
  for (int p = 0; p < n_parts; p++) {
    const int64_t n = parts[p]->d.n;
    const int64_t *ids = node_ids ? node_ids[p] : nullptr;
    for (int64_t c = 0; c < n; c++) {
      const int64_t g = ids ? ids[c] : next + c;
      if (g < 0 || g >= total) return fail(CM_ERR_ARG, "node index " + std::to_string(g) + " out of range");
      if (own[(size_t)g].part >= 0) return fail(CM_ERR_ARG, "node " + std::to_string(g) + " in two parts");
      own[(size_t)g] = Owner{p, c};
    }
    next += n;
  }
  return CM_OK;
}

int copy_vm_in(cm_batch_s *b, const double *Vm, std::vector<double> &out) {
  out.resize((size_t)b->d.n);
  if (b->d.n == 0) return CM_OK;
  if (!Vm) return fail(CM_ERR_ARG, "NULL Vm");
  if (is_device_ptr(Vm)) CK(cudaMemcpy(out.data(), Vm, b->d.n * sizeof(double), cudaMemcpyDeviceToHost));
  else memcpy(out.data(), Vm, b->d.n * sizeof(double));
  return CM_OK;
}

}  // namespace

extern "C" {

int cm_backup_write(const char *path, const char *time_str, int n_parts, const cm_batch_t *parts,
                    const int64_t *const *node_ids, const double *const *Vm) {
  if (!path || !time_str || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  if (!*time_str || strpbrk(time_str, " \t\r\n")) return fail(CM_ERR_ARG, "the time string must be one word");
  std::vector<Owner> own;
  int rc = node_owners(n_parts, parts, node_ids, own);
  if (rc) return rc;
  std::vector<std::vector<double>> blk(n_parts), vm(n_parts);
  for (int p = 0; p < n_parts; p++) {
    cm_batch_s *b = parts[p];
    blk[p].resize((size_t)b->ps.spec->ref_block_doubles * b->d.n);
    if (b->d.n && (rc = cm_batch_get_state(b, CM_LAYOUT_REF_BLOCK, blk[p].data()))) return rc;
    if ((rc = copy_vm_in(b, Vm[p], vm[p]))) return rc;
  }
  FILE *f = fopen(path, "wb");
  if (!f) return fail(CM_ERR_FILE, std::string("cannot open ") + path + " for writing");
  bool ok = fprintf(f, "%s\n%s %lld\n", kBackupVersion, time_str, (long long)own.size()) > 0;
  for (size_t g = 0; ok && g < own.size(); g++) {
    const int p = own[g].part;
    const int64_t c = own[g].local;
    const int nb = parts[p]->ps.spec->ref_block_doubles;
    ok = fwrite(&vm[p][(size_t)c], sizeof(double), 1, f) == 1 &&
         fwrite(&blk[p][(size_t)c * nb], sizeof(double), (size_t)nb, f) == (size_t)nb;
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) return fail(CM_ERR_FILE, std::string("writing ") + path + " failed");
  return CM_OK;
}

int cm_backup_read(const char *path, int n_parts, const cm_batch_t *parts, const int64_t *const *node_ids,
                   double *const *Vm, char *time_out, size_t time_cap) {
  if (!path || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  std::vector<Owner> own;
  int rc = node_owners(n_parts, parts, node_ids, own);
  if (rc) return rc;
  FILE *f = fopen(path, "rb");
  if (!f) return fail(CM_ERR_FILE, std::string("cannot open ") + path);
  // header (acCELLerate.cpp:1543-1566): the version word, then "<time> <nodes>"
  char ver[256] = {0}, line[256] = {0}, ts[64] = {0};
  long long count = -1;
  bool ok = fgets(ver, sizeof ver, f) && fgets(line, sizeof line, f);
  if (ok) {
    const size_t lv = strcspn(ver, "\r\n");
    ver[lv] = 0;
    ok = strcasecmp(ver, kBackupVersion) == 0;
    if (!ok) {
      fclose(f);
      return fail(CM_ERR_FILE, std::string(path) + " is not an acCELLerate backup of version 1.0");
    }
    ok = sscanf(line, "%63s %lld", ts, &count) == 2;
  }
  if (!ok) {
    fclose(f);
    return fail(CM_ERR_FILE, std::string("cannot read the header of ") + path);
  }
  if (count != (long long)own.size()) {
    fclose(f);
    return fail(CM_ERR_FILE, std::string(path) + " holds " + std::to_string(count) + " nodes, the parts " +
                                 std::to_string(own.size()));
  }
  // size check (acCELLerate.cpp:1575-1578): header plus one Vm and one block per node
  const long body = ftell(f);
  long long expect = body;
  for (const Owner &o : own) expect += (long long)(1 + parts[o.part]->ps.spec->ref_block_doubles) * 8;
  fseek(f, 0, SEEK_END);
  const long long size = ftell(f);
  if (size != expect) {
    fclose(f);
    return fail(CM_ERR_FILE, std::string(path) + " has " + std::to_string(size) + " bytes, the parts need " +
                                 std::to_string(expect));
  }
  fseek(f, body, SEEK_SET);
  std::vector<std::vector<double>> blk(n_parts), vm(n_parts);
  for (int p = 0; p < n_parts; p++) {
    blk[p].resize((size_t)parts[p]->ps.spec->ref_block_doubles * parts[p]->d.n);
    vm[p].resize((size_t)parts[p]->d.n);
  }
  for (size_t g = 0; ok && g < own.size(); g++) {
    const int p = own[g].part;
    const int64_t c = own[g].local;
    const int nb = parts[p]->ps.spec->ref_block_doubles;
    ok = fread(&vm[p][(size_t)c], sizeof(double), 1, f) == 1 &&
         fread(&blk[p][(size_t)c * nb], sizeof(double), (size_t)nb, f) == (size_t)nb;
  }
  fclose(f);
  if (!ok) return fail(CM_ERR_FILE, std::string("reading ") + path + " failed");
  for (int p = 0; p < n_parts; p++) {
    cm_batch_s *b = parts[p];
    if (b->d.n == 0) continue;
    if ((rc = cm_batch_set_state(b, CM_LAYOUT_REF_BLOCK, blk[p].data()))) return rc;
    if (!Vm[p]) return fail(CM_ERR_ARG, "NULL Vm");
    if (is_device_ptr(Vm[p]))
      CK(cudaMemcpy(Vm[p], vm[p].data(), b->d.n * sizeof(double), cudaMemcpyHostToDevice));
    else
      memcpy(Vm[p], vm[p].data(), b->d.n * sizeof(double));
  }
  if (time_out && time_cap) {
    strncpy(time_out, ts, time_cap - 1);
    time_out[time_cap - 1] = 0;
  }
  return CM_OK;
}

}  // extern "C"
