/* A plain C caller of the drop-in ABI, as an application linked against libmeshopt_gb300.so in
 * place of libmeshoptimizer would be: it includes only include/meshopt_gb300.h, links only the
 * library, and calls meshopt_simplify / meshopt_simplifyWithAttributes with host buffers.
 *
 *   dropin_cases <cases.txt> <results.txt>
 *
 * cases.txt (whitespace separated; floats as C99 hexadecimal literals, exact):
 *   N, then per case:
 *   name index_count vertex_count stride_bytes position_floats target error options attr_count
 *   attr_stride_bytes attribute_floats has_lock
 *   indices[index_count]
 *   positions[position_floats]
 *   weights[attr_count] attributes[attribute_floats]   (when attr_count > 0; an interleaved array
 *                                                       may end after its last record's used fields)
 *   lock[vertex_count]                                                    (when has_lock)
 *
 * results.txt, per case two lines: the 32-bit call, then the same call made the way a 16-bit
 * index caller goes through the 32-bit entry points (indices widened on the way in and narrowed
 * on the way out, as meshoptimizer.h's meshopt_IndexAdapter does), when every index fits 16 bits:
 *   name bits status count error indices[count]
 */
#include "meshopt_gb300.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static float read_float(FILE* f)
{
	char tok[64];
	if (fscanf(f, "%63s", tok) != 1)
		exit(3);
	return strtof(tok, NULL);
}

static unsigned long read_ulong(FILE* f)
{
	unsigned long v;
	if (fscanf(f, "%lu", &v) != 1)
		exit(3);
	return v;
}

static size_t run(unsigned int* out, const unsigned int* idx, size_t ic, const float* pos, size_t vc, size_t stride, size_t target, float error,
    unsigned int options, const float* attr, size_t attr_stride, const float* weights, size_t ac, const unsigned char* lock, float* err)
{
	if (ac == 0 && lock == NULL)
		return meshopt_simplify(out, idx, ic, pos, vc, stride, target, error, options, err);
	return meshopt_simplifyWithAttributes(out, idx, ic, pos, vc, stride, attr, attr_stride, weights, ac, lock, target, error, options, err);
}

int main(int argc, char** argv)
{
	if (argc != 3)
		return 2;
	FILE* in = fopen(argv[1], "r");
	FILE* res = fopen(argv[2], "w");
	if (!in || !res)
		return 2;
	unsigned long n = read_ulong(in);
	for (unsigned long c = 0; c < n; ++c)
	{
		char name[128];
		if (fscanf(in, "%127s", name) != 1)
			return 3;
		size_t ic = read_ulong(in), vc = read_ulong(in), stride = read_ulong(in), npos = read_ulong(in), target = read_ulong(in);
		float error = read_float(in);
		unsigned int options = (unsigned int)read_ulong(in);
		size_t ac = read_ulong(in), attr_stride = read_ulong(in), nattr = read_ulong(in), has_lock = read_ulong(in);

		unsigned int* idx = malloc((ic + 1) * sizeof(unsigned int));
		unsigned int* out = malloc((ic + 1) * sizeof(unsigned int));
		float* pos = malloc((npos + 1) * sizeof(float));
		float* weights = malloc((ac + 1) * sizeof(float));
		float* attr = malloc((nattr + 1) * sizeof(float));
		unsigned char* lock = has_lock ? malloc(vc + 1) : NULL;
		int narrow = 1;
		for (size_t i = 0; i < ic; ++i)
		{
			idx[i] = (unsigned int)read_ulong(in);
			narrow &= idx[i] < 65536;
		}
		for (size_t i = 0; i < npos; ++i)
			pos[i] = read_float(in);
		if (ac)
		{
			for (size_t i = 0; i < ac; ++i)
				weights[i] = read_float(in);
			for (size_t i = 0; i < nattr; ++i)
				attr[i] = read_float(in);
		}
		if (lock)
			for (size_t i = 0; i < vc; ++i)
				lock[i] = (unsigned char)read_ulong(in);

		float err = -1.f;
		size_t count = run(out, idx, ic, pos, vc, stride, target, error, options, ac ? attr : NULL, attr_stride, ac ? weights : NULL, ac, lock, &err);
		fprintf(res, "%s 32 %d %zu %a", name, meshoptgpu_getLastStatus(), count, err);
		for (size_t i = 0; i < count; ++i)
			fprintf(res, " %u", out[i]);
		fprintf(res, "\n");

		if (narrow)
		{
			/* a 16-bit index buffer: widened to 32 bits for the call, the result narrowed back */
			unsigned short* idx16 = malloc((ic + 1) * sizeof(unsigned short));
			unsigned short* out16 = malloc((ic + 1) * sizeof(unsigned short));
			for (size_t i = 0; i < ic; ++i)
				idx16[i] = (unsigned short)idx[i];
			for (size_t i = 0; i < ic; ++i)
				idx[i] = idx16[i];
			float err16 = -1.f;
			size_t count16 = run(out, idx, ic, pos, vc, stride, target, error, options, ac ? attr : NULL, attr_stride, ac ? weights : NULL, ac, lock, &err16);
			for (size_t i = 0; i < count16; ++i)
				out16[i] = (unsigned short)out[i];
			fprintf(res, "%s 16 %d %zu %a", name, meshoptgpu_getLastStatus(), count16, err16);
			for (size_t i = 0; i < count16; ++i)
				fprintf(res, " %u", (unsigned int)out16[i]);
			fprintf(res, "\n");
			free(idx16);
			free(out16);
		}
		free(idx);
		free(out);
		free(pos);
		free(weights);
		free(attr);
		free(lock);
	}
	fclose(in);
	fclose(res);
	return 0;
}
