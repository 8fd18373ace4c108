classdef GPEtaskSpinorGB300 < GPEtaskSpinor
    %GPEtaskSpinorGB300 - GPEtaskSpinor whose solve_split and get_energy run
    %on a GB300 GPU through libgpe (gpe_mex 'create_spinor' context).
    %
    % Drop-in for GPEtaskSpinor: construct it exactly like
    % GPEtaskSpinor(grid, {V1, V2}); g (2x2), coupling, nlincpl, gamma,
    % decay_rate, Ntotal, n_recalc, Vtd, init_state/current_state ({phi1,
    % phi2}), history and user_callback keep their meaning; solve_split,
    % groundstate_itp and get_energy run on the GPU, with a scalar omega
    % (groundstate_itp: its rotating branch, 2D grids).
    % Single-precision grid axes run the step in complex FP32.
    %
    % UNVERIFIED: no MATLAB was available where this file was written; the
    % library calls it makes are covered by the Python tests of the same ABI.

    properties (Hidden, SetAccess = protected)
        gb300_handle = uint64(0)
        gb300_npts = 0          % values of a stacked [X1(:); X2(:)] array
        gb300_class = 'double'
    end

    methods
        function obj = GPEtaskSpinorGB300(grid, trappot)
            obj@GPEtaskSpinor(grid, trappot);
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
            obj.gb300_npts = 2 * prod(n);
            obj.gb300_handle = gpe_mex('create_spinor', grid.ndims, n, dx, span, obj.gb300_class);
        end

        function delete(obj)
            if obj.gb300_handle ~= 0
                gpe_mex('destroy', obj.gb300_handle);
                obj.gb300_handle = uint64(0);
            end
        end

        function phi = solve_split(task, ddt, niter_inner, niter_outer)
            % @GPEtaskSpinor/solve_split.m semantics, executed by libgpe.
            task.dispstat('', 'init');
            tic;
            task.gb300_push();
            if task.current_iter > 0
                phi = task.current_state;
            else
                phi = task.init_state;
            end
            gpe_mex('set_state', task.gb300_handle, complex(gather([phi{1}(:); phi{2}(:)])));
            timedep = ~isempty(task.Vtd);
            if ~timedep
                gpe_mex('set_potential', task.gb300_handle, ...
                    double(gather([task.Vtrap{1}(:); task.Vtrap{2}(:)])));
            end
            gpe_mex('split', task.gb300_handle, ddt, niter_inner, niter_outer, task, timedep);
            phi = task.current_state;
        end

        function [phi, varargout] = groundstate_itp(task, dt, eps, phi)
            % @GPEtaskSpinor/groundstate_itp.m semantics, executed by libgpe.
            if nargin <= 3
                V = task.getVtotal(0);
                phi = cellfun(@(x) task.grid.normalize(rand(size(V{1}), 'like', V{1}) + ...
                    1i * rand(size(V{1}), 'like', V{1})) ./ sqrt(2), cell(1, 2), 'UniformOutput', false);
            end
            task.gb300_push(true);
            v = task.getVtotal(0);
            gpe_mex('set_potential', task.gb300_handle, double(gather([v{1}(:); v{2}(:)])));
            gpe_mex('set_state', task.gb300_handle, complex(gather([phi{1}(:); phi{2}(:)])));
            [MU, MU2, EE] = gpe_mex('itp', task.gb300_handle, dt, eps, nargout >= 3, nargout >= 4);
            phi = task.gb300_state();
            if nargout >= 2, varargout{1} = MU; end
            if nargout >= 3, varargout{2} = MU2; end
            if nargout >= 4, varargout{3} = EE; end
            task.init_state = phi;
            task.current_state = phi;
        end

        function V = gb300_vtotal(task, time)
            % getVtotal(time) of both components, stacked (called once per block).
            v = task.getVtotal(time);
            V = double(gather([v{1}(:); v{2}(:)]));
        end

        function stop = gb300_step(task, step, time, mu, n)
            % Called by the gateway after each outer step (solve_split.m:115); never stops the run.
            task.ext_callback(task.gb300_state(), step, time, mu, n);
            stop = 0;
        end

        function E = get_energy(task, phi, time)
            % GPEtaskSpinor.m:98-110 on the GPU (V at the current time).
            if nargin < 3
                time = task.current_time;
            end
            if nargin < 2
                phi = task.current_state;
            end
            task.gb300_push();
            v = task.getVtotal(time);
            gpe_mex('set_potential', task.gb300_handle, double(gather([v{1}(:); v{2}(:)])));
            gpe_mex('set_state', task.gb300_handle, complex(gather([phi{1}(:); phi{2}(:)])));
            o = gpe_mex('observables', task.gb300_handle);
            E = o(6);
        end
    end

    methods (Access = protected)
        function gb300_push(task, ~)
            if ~isscalar(task.omega)
                error('gpe:omega', 'libgpe runs GPEtaskSpinor with a scalar omega');
            end
            % the spinor ITP's own iteration cap (groundstate_itp.m:123) in place of itp_max_iter
            gpe_mex('set_params', task.gb300_handle, 0, task.gamma, task.decay_rate, ...
                task.Ntotal, task.mu_init, task.n_recalc, 500000, task.itp_min_iter, ...
                double(task.itp_adjust_stepsize), double(task.omega));
            gpe_mex('set_spinor_params', task.gb300_handle, double(task.g), task.coupling, task.nlincpl);
            n = task.current_n;
            if isempty(n)
                n = 0;
            end
            gpe_mex('set_current', task.gb300_handle, task.current_iter, task.current_time, ...
                task.current_mu, n);
        end

        function phi = gb300_state(task)
            s = gpe_mex('get_state', task.gb300_handle, task.gb300_class, [task.gb300_npts 1]);
            sz = size(task.grid.mesh.x);
            half = task.gb300_npts / 2;
            phi = {reshape(s(1:half), sz), reshape(s(half+1:end), sz)};
            if isa(task.grid.x, 'gpuArray')
                phi = cellfun(@gpuArray, phi, 'UniformOutput', false);
            end
        end
    end
end
