// 4x4 matrix with the operations the EDXRaster core uses: TransformPoint of a
// Vector4 (Shader.h:45) and of a Vector3 (RasterTriangle.h:30-32,
// Renderer.cpp:289), Inverse (Renderer.cpp:88) and product (Renderer.cpp:90).
//
// Convention of this build (EDXUtil's own is unpinned): row-major storage,
// column vectors, p' = M * p.  Each output component is accumulated left to
// right in float, ((m0*x + m1*y) + m2*z) + m3*w, with no fused multiply-add.
// The GPU kernels and the C oracle use the same order.
// Test-infrastructure shim; see EDXPrerequisites.h.
#pragma once

#include "EDXPrerequisites.h"

namespace EDX
{
	class Matrix
	{
	public:
		float m[4][4];

		Matrix()
		{
			for (int i = 0; i < 4; i++)
				for (int j = 0; j < 4; j++)
					m[i][j] = (i == j) ? 1.0f : 0.0f;
		}
		explicit Matrix(const float* rowMajor16)
		{
			for (int i = 0; i < 4; i++)
				for (int j = 0; j < 4; j++)
					m[i][j] = rowMajor16[i * 4 + j];
		}

		friend Matrix operator*(const Matrix& a, const Matrix& b)
		{
			Matrix r;
			for (int i = 0; i < 4; i++)
				for (int j = 0; j < 4; j++)
				{
					float s = a.m[i][0] * b.m[0][j];
					s = s + a.m[i][1] * b.m[1][j];
					s = s + a.m[i][2] * b.m[2][j];
					s = s + a.m[i][3] * b.m[3][j];
					r.m[i][j] = s;
				}
			return r;
		}

		static Vector4 TransformPoint(const Vector4& p, const Matrix& M)
		{
			float o[4];
			for (int i = 0; i < 4; i++)
			{
				float s = M.m[i][0] * p.x;
				s = s + M.m[i][1] * p.y;
				s = s + M.m[i][2] * p.z;
				s = s + M.m[i][3] * p.w;
				o[i] = s;
			}
			return Vector4(o[0], o[1], o[2], o[3]);
		}

		// Point transform with homogeneous divide when the resulting w is not
		// exactly one (for an affine raster matrix w is exactly one).
		static Vector3 TransformPoint(const Vector3& p, const Matrix& M)
		{
			float o[4];
			for (int i = 0; i < 4; i++)
			{
				float s = M.m[i][0] * p.x;
				s = s + M.m[i][1] * p.y;
				s = s + M.m[i][2] * p.z;
				s = s + M.m[i][3];
				o[i] = s;
			}
			if (o[3] == 1.0f)
				return Vector3(o[0], o[1], o[2]);
			return Vector3(o[0] / o[3], o[1] / o[3], o[2] / o[3]);
		}

		// General inverse by Gauss-Jordan elimination with partial pivoting in
		// double, rounded to float.  Used only for the eye position.
		static Matrix Inverse(const Matrix& M)
		{
			double a[4][8];
			for (int i = 0; i < 4; i++)
				for (int j = 0; j < 4; j++)
				{
					a[i][j] = M.m[i][j];
					a[i][j + 4] = (i == j) ? 1.0 : 0.0;
				}
			for (int c = 0; c < 4; c++)
			{
				int piv = c;
				for (int r = c + 1; r < 4; r++)
					if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
				if (piv != c)
					for (int j = 0; j < 8; j++) { double t = a[c][j]; a[c][j] = a[piv][j]; a[piv][j] = t; }
				const double d = a[c][c];
				for (int j = 0; j < 8; j++) a[c][j] /= d;
				for (int r = 0; r < 4; r++)
				{
					if (r == c) continue;
					const double f = a[r][c];
					for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j];
				}
			}
			Matrix r;
			for (int i = 0; i < 4; i++)
				for (int j = 0; j < 4; j++)
					r.m[i][j] = (float)a[i][j + 4];
			return r;
		}
	};
}
