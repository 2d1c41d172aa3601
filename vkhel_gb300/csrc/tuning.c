/*
 * Kernel variant table (the autotuner's output).
 *
 * For every kernel family, degree and job-count bucket the table names the
 * variant the dispatcher launches; vkhel_gb300/autotune.py measures the
 * variants on the GPU and writes the table as text, one "family log_n
 * variant [bucket]" line per entry ('#' starts a comment).  The bucket is the
 * launch's jobs per SM: 0 for at most 1, 1 for at most 2, 2 for at most 4, 3
 * for more (the shapes differ in threads per CTA and so in CTAs per SM, and
 * the job count of a degree class -- instances times limbs -- decides how the
 * last wave fills); a line without a bucket sets all four.  The table is read
 * once per process from $VKHEL_TUNE_TABLE, or, when that is unset, from
 * tuning/gb300.txt beside the package that holds libvkhel.so (found through
 * dladdr).  Missing entries keep the built-in default, variant 0.
 * vkhel_tune_set changes an entry (all buckets) at run time (the autotuner
 * uses it to try each variant).
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"

#define FAMILIES 4
#define DEGREES 32
#define BUCKETS 4

static int g_table[FAMILIES][DEGREES][BUCKETS];
static pthread_once_t g_once = PTHREAD_ONCE_INIT;
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;

static int load_file(const char *path) {
	FILE *f = fopen(path, "r");
	if (!f)
		return -1;
	char line[256];
	int n = 0;
	while (fgets(line, sizeof line, f)) {
		char *hash = strchr(line, '#');
		if (hash)
			*hash = 0;
		unsigned fam, log_n, bucket;
		int var;
		const int got = sscanf(line, "%u %u %d %u", &fam, &log_n, &var, &bucket);
		if (got >= 3 && fam < FAMILIES && log_n < DEGREES && var >= 0) {
			if (got == 4 && bucket >= BUCKETS)
				continue;
			for (unsigned b = 0; b < BUCKETS; b++)
				if (got == 3 || b == bucket)
					g_table[fam][log_n][b] = var;
			n++;
		}
	}
	fclose(f);
	return n;
}

static void init_table(void) {
	const char *env = getenv("VKHEL_TUNE_TABLE");
	if (env) {
		if (*env)
			load_file(env);
		return;
	}
	Dl_info info;
	if (!dladdr((void *) &init_table, &info) || !info.dli_fname)
		return;
	char path[4096];
	snprintf(path, sizeof path, "%s", info.dli_fname);
	char *slash = strrchr(path, '/');
	if (!slash)
		return;
	*slash = 0; /* .../vkhel_gb300/_build */
	slash = strrchr(path, '/');
	if (!slash)
		return;
	*slash = 0; /* .../vkhel_gb300 */
	const size_t len = strlen(path);
	snprintf(path + len, sizeof path - len, "/tuning/gb300.txt");
	load_file(path);
}

static int bucket_of(long njobs, int sms) {
	const long s = sms > 0 ? sms : 1;
	return njobs <= s ? 0 : njobs <= 2 * s ? 1 : njobs <= 4 * s ? 2 : 3;
}

int vkh_variant_jobs(int family, int log_n, long njobs, int sms) {
	pthread_once(&g_once, init_table);
	if (family < 0 || family >= FAMILIES || log_n < 0 || log_n >= DEGREES)
		return 0;
	pthread_mutex_lock(&g_mu);
	const int v = g_table[family][log_n][bucket_of(njobs, sms)];
	pthread_mutex_unlock(&g_mu);
	return v;
}

/* The entry for many jobs (more than 4 per SM), and the flags of family 3. */
int vkh_variant(int family, int log_n) {
	return vkh_variant_jobs(family, log_n, 1L << 40, 1);
}

int vkhel_tune_set(uint32_t family, uint32_t log_n, int32_t variant) {
	pthread_once(&g_once, init_table);
	if (family >= FAMILIES || log_n >= DEGREES || variant < 0)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "tune_set: bad family/log_n/variant");
	pthread_mutex_lock(&g_mu);
	for (int b = 0; b < BUCKETS; b++)
		g_table[family][log_n][b] = variant;
	pthread_mutex_unlock(&g_mu);
	return VKHEL_OK;
}

int vkhel_tune_get(uint32_t family, uint32_t log_n) {
	return vkh_variant((int) family, (int) log_n);
}

int vkhel_tune_load(const char *path) {
	pthread_once(&g_once, init_table);
	if (!path)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "tune_load: NULL path");
	pthread_mutex_lock(&g_mu);
	const int n = load_file(path);
	pthread_mutex_unlock(&g_mu);
	if (n < 0)
		return vkh_fail(NULL, VKHEL_ERR_INVALID_ARGUMENT, "tune_load: cannot read %s", path);
	return VKHEL_OK;
}
