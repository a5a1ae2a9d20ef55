/*
 * CPU harness around the reference's own module host code (test
 * infrastructure only; the product library never links it).
 *
 * The reference's denoise, hilite, demosaic, colour, filmcurv and llap
 * main.c are compiled unmodified from the vkdt tree, one shared object per
 * module (oracle/modules/build.py), against the type-only shim of
 * oracle/modules/shim. This file drives them the way the scheduler drives a
 * chain i-raw -> ... -> sink: module instances with the defaults of their
 * `params` files and the connectors of their `connectors` files, the cfg's
 * param lines applied, modify_roi_out forward, modify_roi_in back from the
 * sink, the forward roi propagation, create_nodes and commit_params
 * (src/pipe/graph-run-modules.h:198-545, 600-760; module instances as
 * src/pipe/module.c:7-110 makes them). It restates those scheduler passes
 * for a linear chain; the modules' callbacks and the connector negotiation
 * (src/pipe/connector.c, compiled in) are the reference's own code.
 *
 * The result is what the scheduler would hand to a device layer: the node
 * list (module and kernel tokens, wd, ht, dp, push constants) and every
 * module's uniform block (committed_param, or param).
 */
#include "modules/api.h"
#include "qvk/qvk.h"

#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

// the device-layer global the module host code reads (colour/main.c reads
// float_atomics_supported); zero: no device features
qvk_t qvk;
// the pipeline global of src/pipe/global.c (nprof's install path reads its home directory)
dt_pipe_global_t dt_pipe;

#define HRN_MAX_MODULES 16
#define HRN_MAX_NODES   512

typedef struct hrn_img_t
{ // i-raw's output metadata (the dt_image_params_t fields the path reads)
  float    black[4], white[4], whitebalance[4];
  uint32_t filters;
  uint32_t crop_aabb[4];
  float    cam_to_rec2020[9];
  float    noise_a, noise_b;
  uint32_t orientation;   // exif orientation (crop's auto rotation reads it)
}
hrn_img_t;

typedef struct hrn_node_t
{
  uint64_t name, kernel;
  int32_t  wd, ht, dp;
  int32_t  module;          // index into the module list (0: the first module after i-raw)
  int32_t  push_size;
  uint8_t  push[256];
}
hrn_node_t;

typedef struct hrn_module_t
{
  uint64_t name, inst;
  int32_t  uniform_size;    // committed_param_size or param_size
  int32_t  param_size;
  uint8_t  uniform[4096];
  uint8_t  param[4096];     // the params after commit_params (colour writes its white back)
  int32_t  out_wd, out_ht;  // roi of the "output" connector
}
hrn_module_t;

static dt_token_t tok(const char *s) { return dt_token(s); }

static int conn_of(const dt_module_t *m, dt_token_t name)
{
  for(int i = 0; i < m->num_connectors; i++) if(m->connector[i].name == name) return i;
  return -1;
}

// ------------------------------------------------------------------ module class from the tree
static int parse_params(const char *dir, const char *name, dt_module_so_t *so)
{ // `params` file: name:type:count:default[:default...] (src/pipe/global.c reads it the same way)
  char fn[1024];
  snprintf(fn, sizeof(fn), "%s/%s/params", dir, name);
  FILE *f = fopen(fn, "rb");
  if(!f) return 0; // no params
  char line[8192];
  int off = 0;
  while(fgets(line, sizeof(line), f))
  {
    char *save = 0;
    char *pn = strtok_r(line, ":\n", &save);
    char *pt = strtok_r(0, ":\n", &save);
    char *pc = strtok_r(0, ":\n", &save);
    if(!pn || !pt || !pc) continue;
    const int cnt = atoi(pc);
    const dt_token_t type = tok(pt);
    const size_t esz = dt_ui_param_type_size(type);
    if(!esz || cnt <= 0) continue;
    dt_ui_param_t *p = calloc(1, sizeof(dt_ui_param_t) + esz * cnt + 16);
    p->name = tok(pn); p->type = type; p->cnt = cnt; p->offset = off;
    if(type == tok("string"))
    {
      char *v = strtok_r(0, "\n", &save);
      if(v) snprintf(p->str, cnt, "%s", v);
    }
    else
    {
      char *v = 0;
      float last = 0.0f;
      for(int i = 0; i < cnt; i++)
      { // fewer defaults than elements repeat the last one
        v = strtok_r(0, ":\n", &save);
        if(v) last = (float)atof(v);
        if(type == tok("float")) p->val[i] = last;
        else p->vali[i] = (int32_t)last;
      }
    }
    off += (int)(esz * cnt);
    so->param[so->num_params++] = p;
    if(so->num_params >= DT_MAX_PARAMS_PER_MODULE) break;
  }
  fclose(f);
  return 0;
}

static int parse_connectors(const char *dir, const char *name, dt_module_so_t *so)
{ // `connectors` file: name:type:chan:format
  char fn[1024];
  snprintf(fn, sizeof(fn), "%s/%s/connectors", dir, name);
  FILE *f = fopen(fn, "rb");
  if(!f) return 1;
  char line[512];
  while(fgets(line, sizeof(line), f) && so->num_connectors < DT_MAX_CONNECTORS)
  {
    char *save = 0;
    char *cn = strtok_r(line, ":\n", &save), *ct = strtok_r(0, ":\n", &save);
    char *cc = strtok_r(0, ":\n", &save), *cf = strtok_r(0, ":\n", &save);
    if(!cn || !ct || !cc || !cf) continue;
    dt_connector_t *c = so->connector + so->num_connectors++;
    memset(c, 0, sizeof(*c));
    c->name = tok(cn); c->type = tok(ct); c->chan = tok(cc); c->format = tok(cf);
  }
  fclose(f);
  return 0;
}

static int load_so(const char *dir, const char *so_dir, const char *name, dt_module_so_t *so)
{
  memset(so, 0, sizeof(*so));
  so->name = tok(name);
  char fn[1024];
  snprintf(fn, sizeof(fn), "%s/mod_%s.so", so_dir, name);
  so->dlhandle = dlopen(fn, RTLD_NOW | RTLD_LOCAL);
  if(!so->dlhandle) { fprintf(stderr, "harness: %s\n", dlerror()); return 1; }
  so->modify_roi_out = (dt_module_modify_roi_out_t)dlsym(so->dlhandle, "modify_roi_out");
  so->modify_roi_in  = (dt_module_modify_roi_in_t) dlsym(so->dlhandle, "modify_roi_in");
  so->create_nodes   = (dt_module_create_nodes_t)  dlsym(so->dlhandle, "create_nodes");
  so->commit_params  = (dt_module_commit_params_t) dlsym(so->dlhandle, "commit_params");
  so->init           = (dt_module_init_t)          dlsym(so->dlhandle, "init");
  so->cleanup        = (dt_module_init_t)          dlsym(so->dlhandle, "cleanup");
  if(parse_params(dir, name, so)) return 1;
  return parse_connectors(dir, name, so);
}

// ------------------------------------------------------------------ module instances (module.c:7-110)
static int module_add(dt_graph_t *g, dt_module_so_t *so, dt_token_t name, dt_token_t inst, uint8_t *pool, int *pool_end)
{
  const int id = g->num_modules++;
  dt_module_t *m = g->module + id;
  memset(m, 0, sizeof(*m));
  m->name = name; m->inst = inst; m->graph = g; m->so = so;
  if(so && so->num_params)
  {
    dt_ui_param_t *p = so->param[so->num_params - 1];
    m->param_size = p->offset + dt_ui_param_size(p->type, p->cnt);
    m->param = pool + *pool_end;
    *pool_end += (m->param_size + 15) & ~15;
    for(int k = 0; k < so->num_params; k++)
      memcpy(m->param + so->param[k]->offset, so->param[k]->val, dt_ui_param_size(so->param[k]->type, so->param[k]->cnt));
  }
  if(so)
  {
    m->num_connectors = so->num_connectors;
    for(int c = 0; c < so->num_connectors; c++)
    {
      m->connector[c] = so->connector[c];
      dt_connector_t *cn = m->connector + c;
      cn->array_length = 1;
      if(cn->type == tok("read") || cn->type == tok("sink") || cn->type == tok("modify")) cn->connected = s_cid_unset;
      else cn->connected = (dt_cid_t){ .i = -1, .c = 0 };   // write/source: no reader yet
      cn->bypass = s_cid_unset;
    }
  }
  return id;
}

static int set_param(dt_module_t *m, const char *pname, const char *vals)
{ // a cfg param line's values
  const int p = dt_module_get_param(m->so, tok(pname));
  if(p < 0) return 1;
  dt_ui_param_t *d = m->so->param[p];
  char buf[8192];
  snprintf(buf, sizeof(buf), "%s", vals);
  if(d->type == tok("string")) { snprintf((char *)m->param + d->offset, d->cnt, "%s", buf); return 0; }
  char *save = 0, *v = strtok_r(buf, ":\n", &save);
  for(int i = 0; i < d->cnt && v; i++, v = strtok_r(0, ":\n", &save))
  {
    if(d->type == tok("float")) ((float *)(m->param + d->offset))[i] = (float)atof(v);
    else ((int32_t *)(m->param + d->offset))[i] = atoi(v);
  }
  return 0;
}

// ------------------------------------------------------------------ scheduler passes (linear chain)
static void pass_roi_out(dt_graph_t *g, dt_module_t *m)
{ // graph-run-modules.h:198-337 modify_roi_out
  const int input = conn_of(m, tok("input"));
  m->img_param = (dt_image_params_t){{0}};
  dt_connector_t *c = input >= 0 ? m->connector + input : 0;
  if(c && c->connected.i >= 0) m->img_param = g->module[c->connected.i].img_param;
  for(int i = 0; i < m->num_connectors; i++)
  { // &input channel references
    dt_connector_t *ci = m->connector + i;
    if(dt_token_str(ci->chan)[0] == '&')
    {
      const dt_token_t ref = ci->chan >> 8;
      for(int j = 0; j < m->num_connectors; j++)
        if(m->connector[j].name == ref) { ci->chan = m->connector[j].chan; break; }
    }
  }
  for(int i = 0; i < m->num_connectors; i++)
  {
    dt_connector_t *ci = m->connector + i;
    if(dt_connector_input(ci) && ci->connected.i >= 0 && ci->connected.c >= 0)
      ci->roi = g->module[ci->connected.i].connector[ci->connected.c].roi;
  }
  if(m->so->modify_roi_out)
  {
    for(int i = 0; i < m->num_connectors; i++)
      if(dt_connector_owner(m->connector + i)) m->connector[i].roi.marker = s_roi_mark_uninited;
    m->so->modify_roi_out(g, m);
    for(int i = 0; i < m->num_connectors; i++)
      if(m->connector[i].roi.marker == s_roi_mark_uninited) m->connector[i].roi.marker = s_roi_mark_soft_fwd;
  }
  else
  {
    dt_roi_t roi = { .marker = s_roi_mark_soft_fwd };
    if(c && c->connected.i != -1) { roi = g->module[c->connected.i].connector[c->connected.c].roi; c->roi = roi; }
    for(int i = 0; i < m->num_connectors; i++)
      if(m->connector[i].type == tok("write"))
      {
        m->connector[i].roi.full_wd = roi.full_wd;
        m->connector[i].roi.full_ht = roi.full_ht;
        m->connector[i].roi.marker = s_roi_mark_soft_fwd;
      }
  }
  for(int i = 0; i < m->num_connectors; i++)
    if(dt_connector_owner(m->connector + i))
    {
      m->connector[i].roi.wd = m->connector[i].roi.full_wd;
      m->connector[i].roi.ht = m->connector[i].roi.full_ht;
    }
}

static void sync_inputs(dt_graph_t *g, dt_module_t *m, int from_roi_in)
{ // graph-run-modules.h:493-545 (from_roi_in) and 348-392: keep input and upstream output rois in sync
  for(int i = 0; i < m->num_connectors; i++)
  {
    dt_connector_t *c = m->connector + i;
    if(!dt_connector_input(c) || dt_cid_unset(c->connected)) continue;
    dt_connector_t *up = &g->module[c->connected.i].connector[c->connected.c];
    dt_roi_t *roi = &up->roi;
    if(from_roi_in && up->type == tok("source"))
    {
      roi->wd = roi->full_wd; roi->ht = roi->full_ht;
      if(roi->marker == s_roi_mark_uninited) roi->marker = s_roi_mark_hard_bck;
      c->roi = *roi;
    }
    if(!from_roi_in && roi->wd == 0)
    {
      if(roi->full_wd == 0) roi->full_wd = 2;
      if(roi->full_ht == 0) roi->full_ht = 2;
      roi->wd = roi->full_wd; roi->ht = roi->full_ht;
      if(roi->marker == s_roi_mark_uninited) roi->marker = s_roi_mark_soft_fwd;
    }
    if(!dt_roi_stronger(&c->roi, roi)) { c->roi = *roi; c->format = up->format; c->chan = up->chan; }
    else { *roi = c->roi; up->format = c->format; up->chan = c->chan; }
    if(from_roi_in) up->flags |= c->flags;
    c->array_length = up->array_length;
  }
}

static void pass_roi_in(dt_graph_t *g, dt_module_t *m)
{ // graph-run-modules.h:448-545 modify_roi_in
  if(m->so->modify_roi_in) m->so->modify_roi_in(g, m);
  else
  {
    const int output = conn_of(m, tok("output"));
    if(output >= 0)
    {
      const dt_roi_t *roi = &m->connector[output].roi;
      for(int i = 0; i < m->num_connectors; i++)
        if(dt_connector_input(m->connector + i)) m->connector[i].roi = *roi;
    }
  }
  sync_inputs(g, m, 1);
}

static void pass_propagate(dt_graph_t *g, dt_module_t *m)
{ // graph-run-modules.h:338-446 propagate_roi_in
  sync_inputs(g, m, 0);
  if(m->so->modify_roi_out)
  {
    dt_module_t tmp = *m;
    for(int i = 0; i < m->num_connectors; i++)
    {
      tmp.connector[i].roi.full_wd = tmp.connector[i].roi.wd;
      tmp.connector[i].roi.full_ht = tmp.connector[i].roi.ht;
    }
    m->so->modify_roi_out(g, &tmp);
    for(int i = 0; i < m->num_connectors; i++)
      if(dt_connector_owner(m->connector + i))
      {
        m->connector[i].roi.wd = tmp.connector[i].roi.full_wd;
        m->connector[i].roi.ht = tmp.connector[i].roi.full_ht;
        m->connector[i].roi.marker = tmp.connector[i].roi.marker;
      }
  }
  else
  {
    const int input = conn_of(m, tok("input"));
    dt_roi_t roi = { 0 };
    if(input >= 0) roi = m->connector[input].roi;
    for(int i = 0; i < m->num_connectors; i++)
      if(m->connector[i].type == tok("write")) { m->connector[i].roi.wd = roi.wd; m->connector[i].roi.ht = roi.ht; }
  }
}

static void pass_create_nodes(dt_graph_t *g, dt_module_t *m)
{ // graph-run-modules.h:33-113: the module's create_nodes, or one node "main" copying the module
  for(int i = 0; i < m->num_connectors; i++) m->connector[i].bypass = s_cid_unset;
  if(m->so->create_nodes) { m->so->create_nodes(g, m); return; }
  const int id = g->num_nodes++;
  dt_node_t *n = g->node + id;
  memset(n, 0, sizeof(*n));
  n->name = m->name; n->kernel = tok("main"); n->num_connectors = m->num_connectors; n->module = m; n->flags = m->flags;
  const int output = conn_of(m, tok("output"));
  if(output >= 0) { n->wd = m->connector[output].roi.wd; n->ht = m->connector[output].roi.ht; n->dp = 1; }
  for(int i = 0; i < m->num_connectors; i++) dt_connector_copy(g, m, i, id, i);
}

// ------------------------------------------------------------------ entry point
/* cfg: the chain's module:/connect:/param: lines (the cfg syntax of
 * src/pipe/graph-io.c); the i-raw:main module is the source, emulated with
 * wd x ht and *img; a sink after the last module asks out_wd x out_ht (0:
 * the full size). Returns 0 and fills the node and module lists. */
int hrn_run(const char *modules_dir, const char *so_dir, const char *cfg, int wd, int ht, const hrn_img_t *img,
    int out_wd, int out_ht, hrn_node_t *nodes, int max_nodes, int *num_nodes, hrn_module_t *mods, int max_mods,
    int *num_mods)
{
  static dt_module_so_t sos[HRN_MAX_MODULES];
  static uint8_t pool[1 << 20];
  int pool_end = 0;
  dt_graph_t *g = calloc(1, sizeof(dt_graph_t));
  g->module = calloc(HRN_MAX_MODULES, sizeof(dt_module_t));
  g->max_modules = HRN_MAX_MODULES;
  g->node = calloc(HRN_MAX_NODES, sizeof(dt_node_t));
  g->max_nodes = HRN_MAX_NODES;
  int nso = 0, r = 0;
  // the source: i-raw:main (i-raw/main.c:138-259 modify_roi_out fills these)
  const int src = module_add(g, 0, tok("i-raw"), tok("main"), pool, &pool_end);
  {
    dt_module_t *m = g->module + src;
    m->num_connectors = 1;
    dt_connector_t *c = m->connector;
    memset(c, 0, sizeof(*c));
    c->name = tok("output"); c->type = tok("source"); c->chan = tok("rggb"); c->format = tok("ui16");
    c->connected = (dt_cid_t){ .i = -1, .c = 0 }; c->bypass = s_cid_unset; c->array_length = 1;
    c->roi = (dt_roi_t){ .full_wd = (uint32_t)wd, .full_ht = (uint32_t)ht, .wd = (uint32_t)wd, .ht = (uint32_t)ht,
                         .marker = s_roi_mark_hard_fwd };
    dt_image_params_t *p = &m->img_param;
    for(int k = 0; k < 4; k++) { p->black[k] = img->black[k]; p->white[k] = img->white[k]; p->whitebalance[k] = img->whitebalance[k]; }
    p->filters = img->filters;
    for(int k = 0; k < 4; k++) p->crop_aabb[k] = img->crop_aabb[k];
    for(int k = 0; k < 9; k++) p->cam_to_rec2020[k] = img->cam_to_rec2020[k];
    p->noise_a = img->noise_a; p->noise_b = img->noise_b;
    p->orientation = img->orientation;
    p->colour_primaries = s_colour_primaries_custom; p->colour_trc = s_colour_trc_linear;
    p->input_name = tok("main");
  }
  // modules, params, connections from the cfg text
  char *text = strdup(cfg);
  char *save = 0;
  for(char *line = strtok_r(text, "\n", &save); line; line = strtok_r(0, "\n", &save))
  {
    char *f[8] = { 0 };
    int n = 0;
    char *ls = 0;
    char *cpy = strdup(line);
    for(char *t = strtok_r(cpy, ":", &ls); t && n < 8; t = strtok_r(0, n == 4 && !strcmp(f[0], "param") ? "\n" : ":", &ls))
      f[n++] = t;
    if(n >= 3 && !strcmp(f[0], "module") && strcmp(f[1], "i-raw"))
    {
      if(nso >= HRN_MAX_MODULES - 1 || load_so(modules_dir, so_dir, f[1], sos + nso)) { r = 1; free(cpy); break; }
      const int id = module_add(g, sos + nso, tok(f[1]), tok(f[2]), pool, &pool_end);
      nso++;
      dt_module_t *m = g->module + id;
      if(m->so->init) m->so->init(m);
    }
    else if(n >= 5 && !strcmp(f[0], "param"))
    {
      for(int i = 1; i < g->num_modules; i++)
        if(g->module[i].name == tok(f[1]) && g->module[i].inst == tok(f[2])) set_param(g->module + i, f[3], f[4]);
    }
    free(cpy);
  }
  free(text);
  if(r) return r;
  text = strdup(cfg);
  for(char *line = strtok_r(text, "\n", &save); line; line = strtok_r(0, "\n", &save))
  { // connect:m0:i0:c0:m1:i1:c1 (graph-io.c)
    char *f[8] = { 0 };
    int n = 0;
    char *ls = 0;
    for(char *t = strtok_r(line, ":", &ls); t && n < 8; t = strtok_r(0, ":", &ls)) f[n++] = t;
    if(n < 7 || strcmp(f[0], "connect")) continue;
    int m0 = -1, m1 = -1;
    for(int i = 0; i < g->num_modules; i++)
    {
      if(g->module[i].name == tok(f[1]) && g->module[i].inst == tok(f[2])) m0 = i;
      if(g->module[i].name == tok(f[4]) && g->module[i].inst == tok(f[5])) m1 = i;
    }
    if(m0 < 0 || m1 < 0) continue;   // a module outside the chain (display, export)
    const int c0 = conn_of(g->module + m0, tok(f[3]));
    const int c1 = conn_of(g->module + m1, tok(f[6]));
    if(c0 < 0 || c1 < 0 || dt_module_connect(g, m0, c0, m1, c1)) { r = 2; break; }
  }
  free(text);
  if(r) return r;
  for(int i = 1; i < g->num_modules; i++)
    if(g->module[i].committed_param_size)
      g->module[i].committed_param = calloc(1, g->module[i].committed_param_size);
  // graph-run-modules.h:641-650, 746-756: roi out, roi in from the sink, propagation, nodes
  const int last = g->num_modules - 1;
  for(int i = 1; i < g->num_modules; i++) pass_roi_out(g, g->module + i);
  { // the sink after the last module (a display or export asks this size, with a scale to fit)
    const int o = conn_of(g->module + last, tok("output"));
    dt_roi_t *roi = &g->module[last].connector[o].roi;
    float scale = 1.0f;
    if(out_wd > 0 && out_ht > 0)
    {
      const float sx = roi->full_wd / (float)out_wd, sy = roi->full_ht / (float)out_ht;
      scale = sx > sy ? sx : sy;
    }
    roi->wd = (uint32_t)(roi->full_wd / scale + 0.5f);
    roi->ht = (uint32_t)(roi->full_ht / scale + 0.5f);
    roi->marker = s_roi_mark_hard_bck;
  }
  for(int i = last; i >= 1; i--) pass_roi_in(g, g->module + i);
  for(int i = 1; i < g->num_modules; i++) pass_propagate(g, g->module + i);
  for(int i = 1; i < g->num_modules; i++) pass_create_nodes(g, g->module + i);
  for(int i = 1; i < g->num_modules; i++)
    if(g->module[i].so->commit_params) g->module[i].so->commit_params(g, g->module + i);
  // results
  *num_nodes = 0;
  for(int i = 0; i < (int)g->num_nodes && *num_nodes < max_nodes; i++)
  {
    const dt_node_t *n = g->node + i;
    hrn_node_t *o = nodes + (*num_nodes)++;
    memset(o, 0, sizeof(*o));
    o->name = n->name; o->kernel = n->kernel; o->wd = n->wd; o->ht = n->ht; o->dp = n->dp;
    o->module = n->module ? (int)(n->module - g->module) - 1 : -1;
    o->push_size = (int32_t)n->push_constant_size;
    memcpy(o->push, n->push_constant, n->push_constant_size > 256 ? 256 : n->push_constant_size);
  }
  *num_mods = 0;
  for(int i = 1; i < g->num_modules && *num_mods < max_mods; i++)
  {
    const dt_module_t *m = g->module + i;
    hrn_module_t *o = mods + (*num_mods)++;
    memset(o, 0, sizeof(*o));
    o->name = m->name; o->inst = m->inst;
    const int us = m->committed_param_size ? (int)m->committed_param_size : (int)m->param_size;
    o->uniform_size = us;
    memcpy(o->uniform, m->committed_param_size ? m->committed_param : m->param, us > 4096 ? 4096 : us);
    o->param_size = (int)m->param_size;
    memcpy(o->param, m->param, m->param_size > 4096 ? 4096 : m->param_size);
    const int oc = conn_of(m, tok("output"));
    if(oc >= 0) { o->out_wd = m->connector[oc].roi.wd; o->out_ht = m->connector[oc].roi.ht; }
  }
  return 0;
}

/* nprof/main.c:82-198 write_sink on a rawhist histogram (3 rows of wd floats:
 * counts, sums of means, sums of second moments): the module writes its fit
 * to "unknown--0.nprof" in the working directory (the image has no maker,
 * model or iso here). Returns 0 when the module ran. */
int hrn_nprof(const char *so_dir, const float *hist, int wd)
{
  char fn[1024];
  snprintf(fn, sizeof(fn), "%s/mod_nprof.so", so_dir);
  void *h = dlopen(fn, RTLD_LAZY | RTLD_LOCAL);
  if(!h) { fprintf(stderr, "harness: %s\n", dlerror()); return 1; }
  dt_module_write_sink_t ws = (dt_module_write_sink_t)dlsym(h, "write_sink");
  if(!ws) return 2;
  dt_module_t *m = calloc(1, sizeof(dt_module_t));
  m->name = tok("nprof"); m->inst = tok("np");
  m->num_connectors = 1;
  m->connector[0].roi.wd = wd; m->connector[0].roi.ht = 5;
  float *buf = calloc((size_t)wd * 5, sizeof(float));
  memcpy(buf, hist, sizeof(float) * 3 * (size_t)wd);
  dt_write_sink_params_t p = { 0 };
  ws(m, buf, &p);
  free(buf);
  free(m);
  return 0;
}
