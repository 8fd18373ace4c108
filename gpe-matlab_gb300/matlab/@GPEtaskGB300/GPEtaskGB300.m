classdef GPEtaskGB300 < GPEtask
    %GPEtaskGB300 - GPEtask whose groundstate_itp and solve_split run on a
    %GB300 GPU through libgpe (gpe_mex MEX gateway).
    %
    % Drop-in for GPEtask: construct it exactly like GPEtask(grid, V); all
    % public properties (g, gamma, decay_rate, Ntotal, mu_init, n_recalc,
    % Vtd, V0, init_state, current_*, history, user_callback, itp_*) keep
    % their meaning.  A grid built from single-precision axes runs the split
    % step in complex FP32 (FP64 reductions); double axes run FP64.
    %
    % UNVERIFIED: no MATLAB was available where this file was written; the
    % library calls it makes are covered by the Python tests of the same ABI.

    properties (Hidden, SetAccess = protected)
        gb300_handle = uint64(0)
        gb300_npts = 0
        gb300_class = 'double'
    end

    methods
        function obj = GPEtaskGB300(grid, trappot)
            obj@GPEtask(grid, trappot);
            x = gather(grid.x);
            y = gather(grid.y);
            obj.gb300_class = class(x);
            if grid.ndims == 3
                z = gather(grid.z);
                n = [numel(x) numel(y) numel(z)];
                dx = double([x(2)-x(1), y(2)-y(1), z(2)-z(1)]);
                span = double([x(end)-x(1), y(end)-y(1), z(end)-z(1)]);
            else
                n = [numel(x) numel(y) 1];
                dx = double([x(2)-x(1), y(2)-y(1), 1]);
                span = double([x(end)-x(1), y(end)-y(1), 0]);
            end
            obj.gb300_npts = prod(n);
            obj.gb300_handle = gpe_mex('create', grid.ndims, n, dx, span, obj.gb300_class);
        end

        function delete(obj)
            if obj.gb300_handle ~= 0
                gpe_mex('destroy', obj.gb300_handle);
                obj.gb300_handle = uint64(0);
            end
        end

        function [phi, varargout] = groundstate_itp(task, dt, eps, phi0)
            % groundstate_itp.m semantics, executed by libgpe.
            if nargin < 4
                phi0 = 'rand';
            end
            task.gb300_push();
            gpe_mex('set_potential', task.gb300_handle, double(gather(task.getVtotal(0))));
            phi = task.process_init_state(phi0);
            task.gb300_put_state(phi);
            [MU, MU2, EE] = gpe_mex('itp', task.gb300_handle, dt, eps, nargout >= 3, nargout >= 4);
            phi = task.gb300_state();
            if nargout >= 2
                varargout{1} = MU;
                if task.Ntotal > 0
                    task.current_mu = MU(end);
                    task.current_n = task.Ntotal;
                end
            end
            if nargout >= 3
                varargout{2} = MU2;
                if task.Ntotal <= 0
                    task.current_mu = MU2(end);
                    task.current_n = MU(end);
                end
            end
            if nargout >= 4
                varargout{3} = EE;
            end
            task.init_state = phi;
            task.current_state = phi;
        end

        function phi = solve_split(task, ddt, niter_inner, niter_outer)
            % solve_split.m semantics, executed by libgpe; ext_callback and
            % user_callback run in MATLAB after every outer step.
            task.dispstat('', 'init');
            tic;
            task.gb300_push();
            if task.current_iter > 0
                phi = task.current_state;
            else
                phi = task.init_state;
            end
            task.gb300_put_state(phi);
            timedep = isa(task.Vtd, 'function_handle') || numel(task.V0) > 1;
            if ~timedep
                gpe_mex('set_potential', task.gb300_handle, double(gather(task.Vtrap)));
            end
            gpe_mex('split', task.gb300_handle, ddt, niter_inner, niter_outer, task, timedep);
            phi = task.current_state;
        end

        function V = gb300_vtotal(task, time)
            % getVtotal(time) as a host double array (called once per block).
            V = double(gather(task.getVtotal(time)));
        end

        function stop = gb300_step(task, step, time, mu, n)
            % Called by the gateway after each outer step (solve_split.m:80);
            % GPEtask ignores the callback's return, so the run never stops here.
            phi = task.gb300_state();
            task.ext_callback(phi, step, time, mu, n);
            stop = 0;
        end

        function [loss, dLdV] = adjoint_grad(task, target, ddt, nsteps, phi0, K, budget, fp64)
            % dloss/dV of loss = 1 - |<target|psi(T)>|^2/(|target|^2 |phi0|^2)
            % after nsteps gamma = 0 split steps from phi0 in Vtrap (GPU discrete
            % adjoint with checkpoints every K steps, K = 0: about sqrt(nsteps)).
            if nargin < 6, K = 0; end
            if nargin < 7, budget = 60e9; end
            if nargin < 8, fp64 = false; end
            task.gb300_push();
            gpe_mex('set_potential', task.gb300_handle, double(gather(task.Vtrap)));
            task.gb300_put_state(phi0);
            [loss, dLdV] = gpe_mex('adjoint', task.gb300_handle, complex(double(gather(target))), ...
                ddt, nsteps, K, budget, 2 * double(fp64));
        end

        function E = get_energy(task, phi, time)
            % GPEtask.m:97-107 on the GPU (current V).
            if nargin >= 2
                task.gb300_put_state(phi);
            end
            o = gpe_mex('observables', task.gb300_handle);
            E = o(6);
        end
    end

    methods (Access = protected)
        function gb300_push(task)
            om = 0;
            if ~isscalar(task.omega)
                % array omega: the Lz Crank-Nicolson branch (ssft_kin_step.m:3-11)
                gpe_mex('set_omega_field', task.gb300_handle, double(gather(task.omega)), task.n_crank);
            else
                gpe_mex('set_omega_field', task.gb300_handle, [], task.n_crank);
                om = double(task.omega);
            end
            gpe_mex('set_params', task.gb300_handle, task.g, task.gamma, task.decay_rate, ...
                task.Ntotal, task.mu_init, task.n_recalc, task.itp_max_iter, task.itp_min_iter, ...
                double(task.itp_adjust_stepsize), om);
            n = task.current_n;
            if isempty(n)
                n = 0;
            end
            gpe_mex('set_current', task.gb300_handle, task.current_iter, task.current_time, ...
                task.current_mu, n);
        end

        function phi = gb300_state(task)
            % gpuArray grids get a gpuArray straight from the device state
            if isa(task.grid.x, 'gpuArray')
                phi = gpe_mex('get_state_gpu', task.gb300_handle, task.gb300_class, size(task.grid.mesh.x));
            else
                phi = gpe_mex('get_state', task.gb300_handle, task.gb300_class, size(task.grid.mesh.x));
            end
        end

        function gb300_put_state(task, phi)
            % a gpuArray state is copied device to device (mxGPUArray), a host one uploaded
            if isa(phi, 'gpuArray')
                gpe_mex('set_state_gpu', task.gb300_handle, complex(phi));
            else
                gpe_mex('set_state', task.gb300_handle, complex(phi));
            end
        end
    end
end
