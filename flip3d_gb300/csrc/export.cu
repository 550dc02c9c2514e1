/*
 * export.cu — the mesh files exporter::write3D writes after a step
 * (src/exporter.cpp:70-167): a Wavefront OBJ (vertices mapped into the unit
 * cube inside the walls, y and z swapped; normals; 1-based faces) and a
 * Sunflow scene (the mesh object with per-vertex normals, vertices clamped
 * to [0.001, 0.999] and scaled by 100). The text is the reference's: the
 * same printf conversions ("%lf", "%d") on the same double expressions, so
 * the files are byte-identical for the same mesh. Formatting runs on host
 * threads, in blocks of lines concatenated in order.
 *
 * flipgpu_export_mesh downloads the device mesh into pinned buffers on the
 * handle's stream and returns; a host thread waits for the copies, formats
 * and writes; flipgpu_export_wait joins it (a new export joins the last).
 */
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "devcommon.cuh"

struct ExportJob {
  std::thread worker;
  int status = FLIPGPU_OK;
  double *V = nullptr, *N = nullptr;
  int32_t *F = nullptr;
  size_t vcap = 0, fcap = 0;
  cudaEvent_t ready = nullptr;
};

namespace {

/* lines [0, count) formatted by line(i, buf) into one string, in blocks on
 * up to 16 host threads */
template <class Line> std::string format_lines(int64_t count, Line line) {
  const int64_t per = 16384;
  const int64_t blocks = (count + per - 1) / per;
  std::vector<std::string> out((size_t)blocks);
  auto run = [&](int64_t b0, int64_t b1) {
    char buf[256];
    for (int64_t b = b0; b < b1; b++) {
      std::string &s = out[(size_t)b];
      s.reserve((size_t)per * 40);
      for (int64_t i = b * per; i < std::min(count, (b + 1) * per); i++) {
        const int len = line(i, buf);
        s.append(buf, (size_t)len);
      }
    }
  };
  const int64_t nt = std::min<int64_t>(blocks, 16);
  if (nt <= 1) {
    run(0, blocks);
  } else {
    std::vector<std::thread> th;
    for (int64_t t = 0; t < nt; t++)
      th.emplace_back(run, blocks * t / nt, blocks * (t + 1) / nt);
    for (auto &x : th) x.join();
  }
  std::string all;
  size_t total = 0;
  for (auto &s : out) total += s.size();
  all.reserve(total);
  for (auto &s : out) all += s;
  return all;
}

bool write_file(const char *path, const std::string &a, const std::string &b = std::string(),
                const std::string &c = std::string()) {
  FILE *fp = fopen(path, "wb");
  if (!fp) return false;
  bool ok = fwrite(a.data(), 1, a.size(), fp) == a.size();
  ok = ok && fwrite(b.data(), 1, b.size(), fp) == b.size();
  ok = ok && fwrite(c.data(), 1, c.size(), fp) == c.size();
  return (fclose(fp) == 0) && ok;
}

/* write_obj (src/exporter.cpp:129-158) */
int obj_file(const char *path, const double *v, const double *n, int64_t nv, const int32_t *f,
             int64_t nf, float wall_thick) {
  const double s = 1.0 / (1.0 - 2.0 * wall_thick);
  const double wt = wall_thick;
  const std::string vs = format_lines(nv, [&](int64_t i, char *buf) {
    return snprintf(buf, 256, "v %lf %lf %lf\n", s * (v[3 * i] - wt), s * (v[3 * i + 2] - wt),
                    s * (v[3 * i + 1] - wt));
  });
  const std::string ns = format_lines(nv, [&](int64_t i, char *buf) {
    return snprintf(buf, 256, "vn %lf %lf %lf\n", n[3 * i], n[3 * i + 2], n[3 * i + 1]);
  });
  const std::string fs = format_lines(nf, [&](int64_t i, char *buf) {
    const int a = f[3 * i] + 1, b = f[3 * i + 1] + 1, c = f[3 * i + 2] + 1;
    return snprintf(buf, 256, "f %d//%d %d//%d %d//%d\n", a, a, b, b, c, c);
  });
  return write_file(path, vs, ns, fs) ? FLIPGPU_OK : FLIPGPU_EINVAL;
}

/* writeSunflow's scene file (src/exporter.cpp:70-127) */
int sunflow_file(const char *path, const double *v, const double *n, int64_t nv,
                 const int32_t *f, int64_t nf, float wall_thick) {
  const double s = 100.0 * 1.0 / (1.0 - 2.0 * wall_thick);
  const double wt = wall_thick;
  const float h = 0.001f;
  char head[256];
  const int hl = snprintf(head, sizeof head,
                          "include template.sc\n\nobject { \n shader Liquid \n type mesh \n name "
                          "polySurfac \n %d %d \n",
                          (int)nv, (int)nf);
  auto clampd = [&](double x) { return fmin(1.0 - h, fmax((double)h, x)); };
  const std::string vs = format_lines(nv, [&](int64_t i, char *buf) {
    return snprintf(buf, 256, "v %lf %lf %lf %lf %lf %lf 0 0\n", s * clampd(v[3 * i] - wt),
                    s * clampd(v[3 * i + 2] - wt), s * clampd(v[3 * i + 1] - wt), n[3 * i],
                    n[3 * i + 2], n[3 * i + 1]);
  });
  std::string fs = format_lines(nf, [&](int64_t i, char *buf) {
    return snprintf(buf, 256, "t %d %d %d\n", f[3 * i], f[3 * i + 1], f[3 * i + 2]);
  });
  fs += "}\n";
  return write_file(path, std::string(head, (size_t)hl), vs, fs) ? FLIPGPU_OK : FLIPGPU_EINVAL;
}

/* mkdir -p */
void make_dir(const std::string &d) {
  for (size_t at = 1; at <= d.size(); at++)
    if (at == d.size() || d[at] == '/') mkdir(d.substr(0, at).c_str(), 0755);
}

} // namespace

int export_join(FlipGpu *h) {
  ExportJob *j = h ? h->exportjob : nullptr;
  if (!j) return FLIPGPU_OK;
  if (j->worker.joinable()) j->worker.join();
  const int r = j->status;
  j->status = FLIPGPU_OK;
  if (r != FLIPGPU_OK)
    snprintf(h->err, sizeof h->err, "export: the mesh download or the file writing failed");
  return r;
}

void export_free(FlipGpu *h) {
  ExportJob *j = h->exportjob;
  if (!j) return;
  export_join(h);
  if (j->V) cudaFreeHost(j->V);
  if (j->N) cudaFreeHost(j->N);
  if (j->F) cudaFreeHost(j->F);
  if (j->ready) cudaEventDestroy(j->ready);
  delete j;
  h->exportjob = nullptr;
}

extern "C" {

int flipgpu_write_obj(const char *path, const double *vertices, const double *normals,
                      int64_t n_vertices, const int32_t *faces, int64_t n_faces,
                      float wall_thick) {
  if (!path || n_vertices < 0 || n_faces < 0 || (n_vertices && (!vertices || !normals)) ||
      (n_faces && !faces))
    return FLIPGPU_EINVAL;
  return obj_file(path, vertices, normals, n_vertices, faces, n_faces, wall_thick);
}

int flipgpu_write_sunflow(const char *path, const double *vertices, const double *normals,
                          int64_t n_vertices, const int32_t *faces, int64_t n_faces,
                          float wall_thick) {
  if (!path || n_vertices < 0 || n_faces < 0 || (n_vertices && (!vertices || !normals)) ||
      (n_faces && !faces))
    return FLIPGPU_EINVAL;
  return sunflow_file(path, vertices, normals, n_vertices, faces, n_faces, wall_thick);
}

int flipgpu_export_mesh(FlipGpu *h, const char *dir, int frame, float wall_thick, int formats,
                        const char *sunflow_template) {
  if (!h || !dir || !(formats & (FLIPGPU_EXPORT_OBJ | FLIPGPU_EXPORT_SUNFLOW)))
    return FLIPGPU_EINVAL;
  export_join(h);
  if (!h->exportjob) h->exportjob = new ExportJob();
  ExportJob *j = h->exportjob;
  int64_t nv = 0, nf = 0;
  if (mesh_download_async(h, nullptr, nullptr, nullptr, &nv, &nf) != FLIPGPU_OK) {
    snprintf(h->err, sizeof h->err, "export_mesh: no mesh (call flipgpu_mesh first)");
    return FLIPGPU_EINVAL;
  }
  if ((size_t)nv > j->vcap) {
    if (j->V) cudaFreeHost(j->V);
    if (j->N) cudaFreeHost(j->N);
    j->V = j->N = nullptr;
    j->vcap = 0;
    if (cudaMallocHost(&j->V, 3 * (size_t)nv * sizeof(double) + 8) != cudaSuccess ||
        cudaMallocHost(&j->N, 3 * (size_t)nv * sizeof(double) + 8) != cudaSuccess)
      return FLIPGPU_ENOMEM;
    j->vcap = (size_t)nv;
  }
  if ((size_t)nf > j->fcap) {
    if (j->F) cudaFreeHost(j->F);
    j->F = nullptr;
    j->fcap = 0;
    if (cudaMallocHost(&j->F, 3 * (size_t)nf * sizeof(int32_t) + 8) != cudaSuccess)
      return FLIPGPU_ENOMEM;
    j->fcap = (size_t)nf;
  }
  if (!j->ready && cudaEventCreateWithFlags(&j->ready, cudaEventDisableTiming) != cudaSuccess)
    return FLIPGPU_ECUDA;
  if (mesh_download_async(h, j->V, j->N, j->F, &nv, &nf) != FLIPGPU_OK ||
      cudaEventRecord(j->ready, h->stream) != cudaSuccess)
    return FLIPGPU_ECUDA;
  const std::string d(dir), tmpl = sunflow_template ? sunflow_template : "";
  const bool has_tmpl = sunflow_template != nullptr;
  j->worker = std::thread([j, d, frame, wall_thick, formats, nv, nf, tmpl, has_tmpl]() {
    if (cudaEventSynchronize(j->ready) != cudaSuccess) {
      j->status = FLIPGPU_ECUDA;
      return;
    }
    int r = FLIPGPU_OK;
    char name[64];
    if (formats & FLIPGPU_EXPORT_OBJ) {
      make_dir(d + "/obj");
      snprintf(name, sizeof name, "/obj/%d_scene.obj", frame);
      r = obj_file((d + name).c_str(), j->V, j->N, nv, j->F, nf, wall_thick);
    }
    if (r == FLIPGPU_OK && (formats & FLIPGPU_EXPORT_SUNFLOW)) {
      make_dir(d + "/sunflow");
      if (has_tmpl && !write_file((d + "/sunflow/template.sc").c_str(), tmpl)) r = FLIPGPU_EINVAL;
      snprintf(name, sizeof name, "/sunflow/%d_scene.sc", frame);
      const std::string fin = d + name, tmp = fin + ".tmp";
      if (r == FLIPGPU_OK) r = sunflow_file(tmp.c_str(), j->V, j->N, nv, j->F, nf, wall_thick);
      if (r == FLIPGPU_OK && rename(tmp.c_str(), fin.c_str()) != 0) r = FLIPGPU_EINVAL;
    }
    j->status = r;
  });
  return FLIPGPU_OK;
}

int flipgpu_export_wait(FlipGpu *h) {
  if (!h) return FLIPGPU_EINVAL;
  return export_join(h);
}

} // extern "C"
