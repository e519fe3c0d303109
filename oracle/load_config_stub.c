/*
 * ORACLE TEST INFRASTRUCTURE -- not the engine.
 *
 * A stand-in for the reference's YAML loader (src/utilities/load_config.c,
 * which needs libyaml, absent here) with the same interface
 * (src/utilities/load_config.h:40,43: load_config / free_config filling
 * ConfigParams).  It reads the subset of YAML that the reference's
 * config.yaml uses: `key: value` scalars (quotes and # comments stripped),
 * a `models:` list of `- name` items and an `indices:` map of
 * `NAME: "file"` items.  It lets the reference's own host program,
 * src/main_runner.c, be built unchanged against the engine's drop-in
 * library in the tests.
 */
#define _POSIX_C_SOURCE 200809L
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "utilities/load_config.h"

static char *trim(char *s)
{
    while (*s && isspace((unsigned char)*s)) s++;
    char *e = s + strlen(s);
    while (e > s && isspace((unsigned char)e[-1])) *--e = '\0';
    return s;
}

/* value without a trailing comment and surrounding quotes */
static char *scalar(char *v)
{
    v = trim(v);
    if (*v == '"' || *v == '\'') {
        const char q = *v++;
        char *end = strchr(v, q);
        if (end) *end = '\0';
        return v;
    }
    char *hash = strchr(v, '#');
    if (hash) *hash = '\0';
    return trim(v);
}

int load_config(const char *filename, ConfigParams *config)
{
    FILE *f = fopen(filename, "r");
    if (!f) {
        fprintf(stderr, "Error: cannot open %s\n", filename);
        return -1;
    }
    memset(config, 0, sizeof(*config));
    char line[1024];
    enum { NONE, MODELS, INDICES } section = NONE;
    while (fgets(line, sizeof line, f)) {
        char *hash = strchr(line, '#');
        const int indented = isspace((unsigned char)line[0]);
        char *s = trim(line);
        if (*s == '\0' || *s == '#') continue;
        (void)hash;
        if (indented && section == MODELS && s[0] == '-') {
            char *name = scalar(s + 1);
            config->models = realloc(config->models, sizeof(char *) * (size_t)(config->num_models + 1));
            config->models[config->num_models++] = strdup(name);
            continue;
        }
        char *colon = strchr(s, ':');
        if (!colon) continue;
        *colon = '\0';
        char *key = trim(s), *val = colon + 1;
        if (indented && section == INDICES) {
            config->indices = realloc(config->indices, sizeof(IndexConfig) * (size_t)(config->num_indices + 1));
            config->indices[config->num_indices].name = strdup(key);
            config->indices[config->num_indices].ticker = strdup(scalar(val));
            config->num_indices++;
            continue;
        }
        section = NONE;
        val = scalar(val);
        if (strcmp(key, "models") == 0) section = MODELS;
        else if (strcmp(key, "indices") == 0) section = INDICES;
        else if (strcmp(key, "start") == 0) config->start = strdup(val);
        else if (strcmp(key, "end") == 0) config->end = strdup(val);
        else if (strcmp(key, "x") == 0) config->x = strtod(val, NULL);
        else if (strcmp(key, "N") == 0) config->N = atoi(val);
        else if (strcmp(key, "M") == 0) config->M = atoi(val);
        else if (strcmp(key, "k") == 0) config->k = atoi(val);
        else if (strcmp(key, "random_seed") == 0) config->random_seed = strtoul(val, NULL, 10);
        else if (strcmp(key, "train_ratio") == 0) config->train_ratio = strtod(val, NULL);
        else if (strcmp(key, "comment") == 0) config->comment = strdup(val);
    }
    fclose(f);
    if (!config->start) config->start = strdup("");
    if (!config->end) config->end = strdup("");
    return 0;
}

void free_config(ConfigParams *config)
{
    if (!config) return;
    free(config->start);
    free(config->end);
    free(config->comment);
    for (int i = 0; i < config->num_indices; i++) {
        free(config->indices[i].name);
        free(config->indices[i].ticker);
    }
    free(config->indices);
    for (int i = 0; i < config->num_models; i++) free(config->models[i]);
    free(config->models);
    memset(config, 0, sizeof(*config));
}
